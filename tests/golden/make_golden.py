"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference checkout exists (FDTD_REFERENCE_ROOT, else the
location oracle/build_ref.py reads), after ``python oracle/build_ref.py``:

    python tests/golden/make_golden.py

Fixtures (seeded random inputs, reference outputs, all in the C-order
(nx, ny, nz) layout of this package, with comparison masks):

  yee_numpy.npz     2nd_order-Yee/Numpy/fdtd3d.py update_e/update_h/pbc,
                    several steps, odd sizes (bit-exact target)
  kemp_core.npz     KEMP/v0.7_pml/fdtd3d/cpu/src/core.c (coeff_use '' and
                    'eh', pad 0..3), one update each, inputs as in
                    KEMP/v0.7_pml/fdtd3d/util/common_random.py:8-39
  cpml_kufdtd.npz   kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c
                    update_{x,y,z}_{e,h}, front and back, remapped to this
                    package's slab layout (kappa = 1), masks cover the cells
                    both conventions update
  symp_c.npz        4th_order-Symplectic/Python-C/dielectric.c update_h /
                    update_e on Fortran-order arrays, compared on
                    [:-1, :-1, :-1] where the C loop bounds and the CUDA
                    index ranges agree
"""
import ctypes as C
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402

REF = build_ref.REF

F32 = np.float32


def _load_module(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def yee_numpy(rng):
    fd = _load_module("ref_fdtd3d", os.path.join(REF, "2nd_order-Yee/Numpy/fdtd3d.py"))
    out = {}
    cases = [((9, 8, 12), 4, 0), ((7, 10, 13), 3, 0), ((5, 6, 7), 5, 0), ((8, 9, 10), 3, 7)]
    for n, (shape, nsteps, pbc_axes) in enumerate(cases):
        names = ["ex", "ey", "ez", "hx", "hy", "hz"]
        f = {k: rng.standard_normal(shape).astype(F32) for k in names}
        ce = [rng.random(shape, dtype=F32) * F32(0.5) for _ in range(3)]
        src = (shape[0] // 2, shape[1] // 2, shape[2] // 2)
        amps = rng.standard_normal(nsteps).astype(F32)
        for k in names:
            out["c%d_in_%s" % (n, k)] = f[k].copy()
        for q, k in enumerate(("cex", "cey", "cez")):
            out["c%d_in_%s" % (n, k)] = ce[q]
        out["c%d_amps" % n] = amps
        out["c%d_src" % n] = np.array(src)
        out["c%d_meta" % n] = np.array([nsteps, pbc_axes])
        dirs = "".join(a for b, a in ((1, "x"), (2, "y"), (4, "z")) if pbc_axes & b)
        for t in range(nsteps):
            fd.update_e(f["ex"], f["ey"], f["ez"], f["hx"], f["hy"], f["hz"], *ce)
            if dirs:
                fd.update_pbc_e(dirs, f["ex"], f["ey"], f["ez"])
            f["ez"][src] += amps[t]
            fd.update_h(f["ex"], f["ey"], f["ez"], f["hx"], f["hy"], f["hz"])
            if dirs:
                fd.update_pbc_h(dirs, f["hx"], f["hy"], f["hz"])
        for k in names:
            out["c%d_out_%s" % (n, k)] = f[k]
    out["ncases"] = np.array(len(cases))
    return out


def kemp_core(rng):
    out = {}
    n = 0
    nx, ny = 6, 7
    for coeff_use in ("", "eh"):
        for nz in (13, 14, 15, 16):
            pad = (-nz) % 4
            lib = np.ctypeslib.load_library(os.path.basename(build_ref.kemp_lib_path(coeff_use, pad)),
                                            os.path.dirname(build_ref.kemp_lib_path(coeff_use, pad)))
            for ufunc in ("e", "h"):
                shape = (nx, ny, nz)
                pitch = (nx, ny, nz + pad)
                if ufunc == "e":
                    ehs = [np.zeros(shape, F32) for _ in range(3)] + [rng.random(shape, dtype=F32) for _ in range(3)]
                else:
                    ehs = [rng.random(shape, dtype=F32) for _ in range(3)] + [np.zeros(shape, F32) for _ in range(3)]
                if coeff_use:
                    ces = [rng.random(shape, dtype=F32) for _ in range(3)]
                    chs = [rng.random(shape, dtype=F32) for _ in range(3)]
                else:
                    ces = [np.full(shape, 0.5, F32) for _ in range(3)]
                    chs = [np.full(shape, 0.5, F32) for _ in range(3)]
                pe = [np.zeros(pitch, F32) for _ in range(6)]
                for a, b in zip(pe, ehs):
                    a[:, :, :nz] = b
                pce = [np.zeros(pitch, F32) for _ in range(3)]
                pch = [np.zeros(pitch, F32) for _ in range(3)]
                for a, b in zip(pce, ces):
                    a[:, :, :nz] = b
                for a, b in zip(pch, chs):
                    a[:, :, :nz] = b
                args = [C.c_int(nx), C.c_int(ny), C.c_int(nz + pad)] + [C.c_void_p(a.ctypes.data) for a in pe]
                if ufunc == "e":
                    if coeff_use:
                        args += [C.c_void_p(a.ctypes.data) for a in pce]
                    lib.update_e(*args)
                else:
                    if coeff_use:
                        args += [C.c_void_p(a.ctypes.data) for a in pch]
                    lib.update_h(*args)
                tag = "c%d_" % n
                out[tag + "meta"] = np.array([nz, pad, 1 if coeff_use else 0, 0 if ufunc == "e" else 1])
                for q, k in enumerate(["ex", "ey", "ez", "hx", "hy", "hz"]):
                    out[tag + "in_" + k] = ehs[q]
                    out[tag + "out_" + k] = pe[q][:, :, :nz].copy()
                for q, k in enumerate(["cex", "cey", "cez"]):
                    out[tag + "in_" + k] = ces[q]
                for q, k in enumerate(["chx", "chy", "chz"]):
                    out[tag + "in_" + k] = chs[q]
                n += 1
    out["ncases"] = np.array(n)
    return out


def cpml_kufdtd(rng):
    """Run the reference's non-kappa CPML routines and remap to the slab layout."""
    sys.path.insert(0, build_ref.OUT)
    import ref_cpml_non_kappa as ref
    out = {}
    n = 0
    Nx, Ny, Nz, P = 9, 8, 12, 3     # Npml+1 multiple of 4 for the z routines
    shape = (Nx, Ny, Nz)
    for axis in range(3):
        for which in ("e", "h"):
            for backward in (0, 1):
                E = [rng.standard_normal(shape).astype(F32) for _ in range(3)]
                H = [rng.standard_normal(shape).astype(F32) for _ in range(3)]
                CE = [rng.random(shape, dtype=F32) for _ in range(3)]
                rb = rng.random(2 * (P + 1), dtype=F32)
                ra = (rng.random(2 * (P + 1), dtype=F32) - F32(0.5))
                if axis == 0:
                    kshape = (P, Ny - 1, Nz)
                elif axis == 1:
                    kshape = (Nx - 1, P, Nz)
                else:
                    kshape = (Nx - 1, Ny - 1, P + 1)
                kpsi = [rng.standard_normal(kshape).astype(F32) for _ in range(2)]
                if axis == 2:       # the kpml=0 / k=Nz-1 planes are outside this package's slabs
                    for p in kpsi:
                        p[:, :, 0 if backward == 0 else P] = 0
                ex, ey, ez = [a.copy() for a in E]
                hx, hy, hz = [a.copy() for a in H]
                kp = [p.copy() for p in kpsi]
                fn = getattr(ref, "update_%s_%s" % ("xyz"[axis], which))
                if which == "e":
                    flds = {0: (ey, ez, hy, hz, CE[1], CE[2]), 1: (ex, ez, hx, hz, CE[0], CE[2]),
                            2: (ex, ey, hx, hy, CE[0], CE[1])}[axis]
                else:
                    flds = {0: (ey, ez, hy, hz), 1: (ex, ez, hx, hz), 2: (ex, ey, hx, hy)}[axis]
                fn(1, Nx, Ny, Nz, P, backward, *flds, kp[0], kp[1], rb, ra)
                # remap: tables and psi into the slab layout (2P entries)
                if which == "e":
                    tb, ta = rb[1:2 * P + 1], ra[1:2 * P + 1]
                else:
                    tb = np.concatenate([rb[1:P + 1], rb[P + 2:2 * P + 2]])
                    ta = np.concatenate([ra[1:P + 1], ra[P + 2:2 * P + 2]])
                n_ax = shape[axis]
                sl = np.arange(P) if backward == 0 else np.arange(P, 2 * P)
                if which == "e":
                    nodes = [s + 1 if s < P else n_ax - P - 1 + (s - P) for s in sl]
                else:
                    nodes = [s + 1 if s < P else n_ax - P + (s - P) for s in sl]
                mshape = [(2 * P, Ny, Nz), (Nx, 2 * P, Nz), (Nx, Ny, 2 * P)][axis]
                psi_in = [np.zeros(mshape, F32) for _ in range(2)]
                psi_out = [np.zeros(mshape, F32) for _ in range(2)]
                pmask = np.zeros(mshape, bool)
                for q, (s, node) in enumerate(zip(sl, nodes)):
                    ip = q  # reference slab plane index (ipml/jpml) or kpml
                    for r in range(2):
                        if axis == 0:
                            psi_in[r][s, 1:, :] = kpsi[r][ip]
                            psi_out[r][s, 1:, :] = kp[r][ip]
                        elif axis == 1:
                            flat_in = kpsi[r].reshape(-1).reshape(P, Nx - 1, Nz)
                            flat_out = kp[r].reshape(-1).reshape(P, Nx - 1, Nz)
                            psi_in[r][1:, s, :] = flat_in[ip]
                            psi_out[r][1:, s, :] = flat_out[ip]
                        else:
                            kp_idx = node - (0 if backward == 0 else Nz - P - 1)
                            psi_in[r][1:, 1:, s] = kpsi[r][:, :, kp_idx]
                            psi_out[r][1:, 1:, s] = kp[r][:, :, kp_idx]
                # comparison region: transverse interior, both conventions update it
                fmask = np.zeros(shape, bool)
                for s, node in zip(sl, nodes):
                    if axis == 0:
                        fmask[node, 1:Ny - 1, 1:Nz - 1] = True
                        pmask[s, 1:Ny - 1, 1:Nz - 1] = True
                    elif axis == 1:
                        fmask[1:Nx - 1, node, 1:Nz - 1] = True
                        pmask[1:Nx - 1, s, 1:Nz - 1] = True
                    else:
                        fmask[1:Nx - 1, 1:Ny - 1, node] = True
                        pmask[1:Nx - 1, 1:Ny - 1, s] = True
                tag = "c%d_" % n
                out[tag + "meta"] = np.array([axis, 0 if which == "e" else 1, backward, P])
                for q, k in enumerate(("ex", "ey", "ez")):
                    out[tag + "in_" + k] = E[q]
                    out[tag + "out_" + k] = [ex, ey, ez][q]
                for q, k in enumerate(("hx", "hy", "hz")):
                    out[tag + "in_" + k] = H[q]
                    out[tag + "out_" + k] = [hx, hy, hz][q]
                for q, k in enumerate(("cex", "cey", "cez")):
                    out[tag + "in_" + k] = CE[q]
                out[tag + "tb"] = tb
                out[tag + "ta"] = ta
                out[tag + "psi_in0"], out[tag + "psi_in1"] = psi_in
                out[tag + "psi_out0"], out[tag + "psi_out1"] = psi_out
                out[tag + "fmask"] = fmask
                out[tag + "pmask"] = pmask
                n += 1
    out["ncases"] = np.array(n)
    out["shape"] = np.array(shape)
    return out


def symp_c(rng):
    sys.path.insert(0, build_ref.OUT)
    import ref_symp_dielectric as ref
    out = {}
    n = 0
    for shape in ((9, 8, 10), (7, 11, 9)):
        nx, ny, nz = shape
        for which in ("h", "e"):
            coef = F32(rng.standard_normal())
            f = [np.asfortranarray(rng.standard_normal(shape).astype(F32)) for _ in range(6)]
            c = [np.asfortranarray(rng.random(shape, dtype=F32)) for _ in range(3)]
            ins = [np.ascontiguousarray(a) for a in f]
            if which == "h":
                ref.update_h(nx, ny, nz, float(coef), *f, *c)
            else:
                ref.update_e(nx, ny, nz, float(coef), *f, *c)
            tag = "c%d_" % n
            out[tag + "meta"] = np.array([0 if which == "h" else 1])
            out[tag + "coef"] = np.array(coef, F32)
            for q, k in enumerate(("ex", "ey", "ez", "hx", "hy", "hz")):
                out[tag + "in_" + k] = ins[q]
                out[tag + "out_" + k] = np.ascontiguousarray(f[q])
            for q, k in enumerate(("c0", "c1", "c2")):
                out[tag + "in_" + k] = np.ascontiguousarray(c[q])
            n += 1
    out["ncases"] = np.array(n)
    return out


def drude_kufdtd(rng):
    """kuFDTD drude_ade.update_e (kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c) on a
    sub-box of the E arrays, three calls in a row (J carries over)."""
    sys.path.insert(0, build_ref.OUT)
    import ref_drude_ade as ref
    import oracle
    out = {}
    n = 0
    # (full grid, box origin, box shape); the reference's k loop takes 4 cells at a time
    for shape, org, box in (((9, 10, 13), (2, 3, 4), (4, 5, 8)), ((6, 7, 12), (0, 0, 0), (6, 7, 12))):
        nx, ny, nz = shape
        E = [rng.standard_normal(shape).astype(F32) for _ in range(3)]
        CE = [rng.random(shape, dtype=F32) for _ in range(3)]
        J = [(0.1 * rng.standard_normal(box)).astype(F32) for _ in range(3)]
        CA, CB = [], []
        for _ in range(3):
            a, b = oracle.drude_coefficients(rng.uniform(0.05, 0.4, box).astype(F32),
                                             rng.uniform(0.0, 0.2, box).astype(F32))
            CA.append(a)
            CB.append(b)
        tag = "c%d_" % n
        out[tag + "meta"] = np.array([*org, *box])
        for q, k in enumerate(("ex", "ey", "ez")):
            out[tag + "in_" + k] = E[q].copy()
            out[tag + "in_c" + k] = CE[q]
            out[tag + "in_j" + k[1]] = J[q].copy()
            out[tag + "in_cja" + k[1]] = CA[q]
            out[tag + "in_cjb" + k[1]] = CB[q]
        idx0 = (org[0] * ny + org[1]) * nz + org[2]
        for _ in range(3):
            ref.update_e(1, box[0], box[1], box[2], idx0, ny * nz, nz, *E, *CE, *J, *CA, *CB)
        for q, k in enumerate(("ex", "ey", "ez")):
            out[tag + "out_" + k] = E[q]
            out[tag + "out_j" + k[1]] = J[q]
        n += 1
    out["ncases"] = np.array(n)
    return out


def _reference_tfsf_module():
    """kuFDTD/v0.2.0/dim3/tfsf.py executed in place under Python 3: its
    imports (kufdtd.common: scipy as sc, light_velocity) are provided by a stub
    module, and three Python-2 idioms are mapped when the text is compiled
    (xrange -> range, `is` between strings -> ==, list indices -> tuples)."""
    import types
    common = types.ModuleType("kufdtd.common")

    class SC:
        zeros = staticmethod(np.zeros)
        sin = staticmethod(np.sin)
        cos = staticmethod(np.cos)
        sqrt = staticmethod(np.sqrt)
        newaxis = None
        pi = np.pi
    common.sc = SC
    common.light_velocity = 2.99792458e8
    pkg = types.ModuleType("kufdtd")
    pkg.common = common
    sys.modules.setdefault("kufdtd", pkg)
    sys.modules.setdefault("kufdtd.common", common)
    path = os.path.join(build_ref.REF, "kuFDTD/v0.2.0/dim3/tfsf.py")
    src = open(path).read()
    src = src.replace("from kufdtd.common import *", "from kufdtd.common import sc, light_velocity")
    src = src.replace(" is '", " == '").replace("' is ", "' == ").replace("[s.sl_expand]", "[tuple(s.sl_expand)]")
    ns = {"xrange": range}
    exec(compile(src, path, "exec"), ns)
    return ns


def tfsf_kufdtd(rng):
    """kuFDTD Tfsf.updateE/updateH from zero fields (no 3-D update in between,
    so only face cells change), polarisation angle 0 (coefficients 0 and +-1:
    the result does not depend on the NumPy version's scalar casting), every
    propagation axis, all faces and a subset."""
    ns = _reference_tfsf_module()

    class Space:
        pass
    out = {}
    n = 0
    shape = (18, 16, 14)
    for axis in "xyz":
        for apply in (("fb", "fb", "fb"), ("f", "b", "fb")):
            S = Space()
            S.Nx, S.Ny, S.Nz = shape
            S.dx = 1.0
            S.dt = 0.5 / 2.99792458e8          # w dt = 2 pi 0.5 / wavelength (in cells)
            f0 = {k: np.zeros(shape, F32) for k in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
            for k, v in f0.items():
                setattr(S, k, v.copy())
            T = ns["Tfsf"]((5, 4, 3), (12, 11, 10), apply, 10.0, ["normal", axis], 0.0)
            T.set_space(S)
            for t in range(1, 13):
                T.updateE(t)
                T.updateH()
            tag = "c%d_" % n
            out[tag + "meta"] = np.array(["xyz".index(axis)] + [int("f" in a) * 1 + int("b" in a) * 2 for a in apply])
            for k in f0:
                out[tag + "out_" + k.lower()] = getattr(S, k)
            out[tag + "e1d"] = T.space1d.E
            out[tag + "h1d"] = T.space1d.H
            n += 1
    out["ncases"] = np.array(n)
    out["pt"] = np.array([[5, 4, 3], [12, 11, 10]])
    out["wdt"] = np.array(2 * np.pi * 2.99792458e8 / 10.0 * (0.5 / 2.99792458e8))
    return out


def output_kufdtd(rng):
    """kuFDTD Output.get_data() (kuFDTD/v0.2.0/dim3/output.py, executed in place
    with the same stub module as the TFSF case) for every dataform on a region
    with a spatial step, and on a plane (pt1 == pt2 on one axis)."""
    import types
    common = types.ModuleType("kufdtd.common")

    class SC:
        sqrt = staticmethod(np.sqrt)
    common.sc = SC

    def list_replace(lst, index, content):       # kuFDTD/v0.2.0/common.py:32-39
        out = list(lst)
        out[index] = content
        return out
    common.list_replace = list_replace
    pkg = types.ModuleType("kufdtd")
    pkg.common = common
    saved = {k: sys.modules.get(k) for k in ("kufdtd", "kufdtd.common")}
    sys.modules["kufdtd"], sys.modules["kufdtd.common"] = pkg, common
    path = os.path.join(build_ref.REF, "kuFDTD/v0.2.0/dim3/output.py")
    src = open(path).read().replace("from kufdtd.common import *", "from kufdtd.common import sc, list_replace")
    src = src.replace("[s.data_slice]", "[tuple(s.data_slice)]").replace("[ e_sl[0] ]", "[ tuple(e_sl[0]) ]")
    src = src.replace("[ e_sl[1] ]", "[ tuple(e_sl[1]) ]")
    for q in range(4):
        src = src.replace("[ h_sl[%d] ]" % q, "[ tuple(h_sl[%d]) ]" % q)
    ns = {"xrange": range}
    exec(compile(src, path, "exec"), ns)
    for k, v in saved.items():
        if v is None:
            sys.modules.pop(k, None)
        else:
            sys.modules[k] = v

    class Space:
        pass
    shape = (12, 11, 10)
    S = Space()
    S.Nx, S.Ny, S.Nz = shape
    f = {k: rng.standard_normal(shape).astype(F32) for k in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
    for k, v in f.items():
        setattr(S, k, v)
    out = {"in_" + k.lower(): v for k, v in f.items()}
    n = 0
    forms = ns["Output"]("e", (1, 1, 1), (2, 2, 2)).__class__   # the class, for the form list below
    for dform in ("e", "e2", "ex", "ey", "ez", "ex2", "ey2", "ez2", "h", "h2", "hx", "hy", "hz", "hx2", "hy2",
                  "hz2", "s", "s2", "sx", "sy", "sz", "sx2", "sy2", "sz2"):
        for pt1, pt2, step in (((2, 1, None), (9, None, 8), (2, 1, 3)), ((None, 4, 2), (None, 4, 8), (1, 1, 2))):
            o = forms(dform, pt1, pt2, step)
            o.set_space(S)
            tag = "c%d_" % n
            out[tag + "form"] = np.array(dform)
            out[tag + "pts"] = np.array([[-1 if v is None else v for v in pt1], [-1 if v is None else v for v in pt2],
                                        list(step)])
            out[tag + "out"] = np.asarray(o.get_data(), dtype=F32)
            n += 1
    out["ncases"] = np.array(n)
    return out


def cpml_kappa_kufdtd(rng):
    """Run the reference's kappa CPML (update_cpml_3d of
    kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c:22-330) and remap it to
    this package's slab layout.  That code keeps E on 'in_field' arrays (one
    cell smaller) and H on 'out_field' arrays (a ghost layer at index 0), the
    'hfaced' grid of boundary/cpml.py:150-158, whose differences are this
    package's (E: forward, H: backward).  Mapping, per face axis d:
      E update (in_field, N[d] = n_d - 3, other N = n - 1): reference cell
        idx <-> our E cell idx + 1 along d; its base H(idx + 1 off d, idx along d)
        <-> our H(idx) shifted by -1 along d; psi and coefficient index equal.
      H update (out_field, N = n - 1): reference cell idx <-> our H cell idx;
        its base E(idx - 1 off d) <-> our E(idx); psi index equal.
    Tables: b, a (FP32) and kappa = 1/(1 + km1) (FP32) from the FP64 tables
    of this package's formula (kappa_max = 5, R = 1e-8, m = 4, alpha_max = 0.05),
    ds = 1.  The H coefficient is the scalar 0.5 (1x1x1 arrays, EorH = -1);
    E takes per-cell coefficient arrays (EorH = +1)."""
    sys.path.insert(0, build_ref.OUT)
    import ref_cpml_core as ref
    import oracle
    out = {}
    n = 0
    shape = (10, 9, 12)
    P = 3
    tab64 = oracle.cpml_tables(P)
    for axis in range(3):
        for which in ("e", "h"):
            for side in ("front", "back"):
                nshape = list(shape)
                perm1, perm2 = (axis + 1) % 3, (axis + 2) % 3
                kapa = (1.0 / (1.0 + tab64["km1_" + which])).astype(F32)
                b = tab64["b_" + which].astype(F32)
                a = tab64["a_" + which].astype(F32)
                if which == "e":
                    N = [v - 1 for v in shape]
                    N[axis] = shape[axis] - 3
                    ushape = [v + 1 for v in N]                 # in_field
                    bshape = [v + 2 for v in N]                 # out_field
                    up = [rng.standard_normal(ushape).astype(F32) for _ in range(3)]
                    base = [rng.standard_normal(bshape).astype(F32) for _ in range(3)]
                    cb = [(rng.random(ushape, dtype=F32) * F32(0.5) + F32(0.05)) for _ in range(3)]
                    pshape = list(ushape)
                    pshape[axis] = 2 * P
                else:
                    N = [v - 1 for v in shape]
                    ushape = [v + 2 for v in N]                 # out_field
                    bshape = [v + 1 for v in N]                 # in_field
                    up = [rng.standard_normal(ushape).astype(F32) for _ in range(3)]
                    base = [rng.standard_normal(bshape).astype(F32) for _ in range(3)]
                    cb = [np.full((1, 1, 1), 0.5, F32) for _ in range(3)]
                    pshape = list(ushape)
                    pshape[axis] = 2 * P
                psi = [None] * 6
                psi[2 * axis] = rng.standard_normal(pshape).astype(F32) * F32(0.1)
                psi[2 * axis + 1] = rng.standard_normal(pshape).astype(F32) * F32(0.1)
                for q in range(6):  # the other axes' psi arrays are not read
                    if psi[q] is None:
                        psi[q] = np.zeros((1, 1, 1), F32)
                up_in = [u.copy() for u in up]
                psi_in = [psi[2 * axis].copy(), psi[2 * axis + 1].copy()]
                ref.update_cpml_3d("in_field" if which == "e" else "out_field", tuple(N), up, base, cb, 1.0, P,
                                   [kapa, b, a], psi, axis, side)
                # ---- remap into this package's layout
                sl_all = [slice(None)] * 3
                ours_up_in, ours_up_out, ours_base, ours_c = [], [], [], []
                for q in range(3):
                    if which == "e":
                        fi = rng.standard_normal(shape).astype(F32)
                        fo = fi.copy()
                        dst = list(sl_all)
                        dst[axis] = slice(1, shape[axis] - 1)
                        fi[tuple(dst)] = up_in[q]
                        fo[tuple(dst)] = up[q]
                        hb = rng.standard_normal(shape).astype(F32)
                        src = [slice(1, shape[x] + 1) for x in range(3)]
                        src[axis] = slice(0, shape[axis] - 1)
                        dsth = list(sl_all)
                        dsth[axis] = slice(1, None)
                        hb[tuple(dsth)] = base[q][tuple(src)]
                        c = (rng.random(shape, dtype=F32) * F32(0.5) + F32(0.05))
                        c[tuple(dst)] = cb[q]
                        ours_c.append(c)
                    else:
                        fi = up_in[q][:shape[0], :shape[1], :shape[2]].copy()
                        fo = up[q][:shape[0], :shape[1], :shape[2]].copy()
                        hb = rng.standard_normal(shape).astype(F32)
                        dst = [slice(1, None)] * 3
                        dst[axis] = slice(None)
                        src = [slice(0, shape[x] - 1) for x in range(3)]
                        src[axis] = slice(None)
                        hb[tuple(dst)] = base[q][tuple(src)]
                    ours_up_in.append(fi)
                    ours_up_out.append(fo)
                    ours_base.append(hb)
                mshape = [shape[0], shape[1], shape[2]]
                mshape[axis] = 2 * P
                crop = tuple(slice(0, v) for v in mshape)
                p_in = [psi_in[r][crop].copy() for r in range(2)]
                p_out = [psi[2 * axis + r][crop].copy() for r in range(2)]
                # comparison masks: the face's nodes, where both conventions update
                nodes = range(1, P + 1) if side == "front" else (
                    range(shape[axis] - P - 1, shape[axis] - 1) if which == "e" else range(shape[axis] - P, shape[axis]))
                fmask = [np.zeros(shape, bool) for _ in range(3)]
                pmask = [np.zeros(mshape, bool) for _ in range(2)]
                for r, comp in enumerate((perm1, perm2)):
                    m = np.zeros(shape, bool)
                    idx = list(sl_all)
                    idx[axis] = list(nodes)
                    m[tuple(idx)] = True
                    for x in range(3):          # the component's own update range
                        if x == comp:
                            continue
                        cut = [slice(None)] * 3
                        if which == "e":
                            cut[x] = shape[x] - 1   # E: the last plane across is never updated
                        else:
                            cut[x] = 0              # H: index 0 is never updated
                        m[tuple(cut)] = False
                    if which == "h":              # the reference's out_field loops start at 1
                        for x in range(3):
                            if x != axis:
                                cut = [slice(None)] * 3
                                cut[x] = 0
                                m[tuple(cut)] = False
                    fmask[comp] = m
                    pm = np.zeros(mshape, bool)
                    s0 = 0 if side == "front" else P
                    idx = list(sl_all)
                    idx[axis] = slice(s0, s0 + P)
                    mm = np.moveaxis(m, axis, 0)[list(nodes)]
                    pm_view = np.moveaxis(pm, axis, 0)
                    pm_view[s0:s0 + P] = mm
                    pmask[r] = pm
                tag = "c%d_" % n
                out[tag + "meta"] = np.array([axis, 0 if which == "e" else 1, 0 if side == "front" else 1, P])
                names_u = ("ex", "ey", "ez") if which == "e" else ("hx", "hy", "hz")
                names_b = ("hx", "hy", "hz") if which == "e" else ("ex", "ey", "ez")
                for q in range(3):
                    out[tag + "in_" + names_u[q]] = ours_up_in[q]
                    out[tag + "out_" + names_u[q]] = ours_up_out[q]
                    out[tag + "in_" + names_b[q]] = ours_base[q]
                    out[tag + "fmask_" + names_u[q]] = fmask[q]
                    if which == "e":
                        out[tag + "in_" + ("cex", "cey", "cez")[q]] = ours_c[q]
                for r in range(2):
                    out[tag + "psi_in%d" % r] = p_in[r]
                    out[tag + "psi_out%d" % r] = p_out[r]
                    out[tag + "pmask%d" % r] = pmask[r]
                out[tag + "tb"] = b
                out[tag + "ta"] = a
                out[tag + "tkm1"] = tab64["km1_" + which].astype(F32)
                n += 1
    out["ncases"] = np.array(n)
    out["shape"] = np.array(shape)
    return out


CASES = (("yee_numpy", yee_numpy), ("kemp_core", kemp_core), ("cpml_kufdtd", cpml_kufdtd), ("symp_c", symp_c),
         ("drude_kufdtd", drude_kufdtd), ("tfsf_kufdtd", tfsf_kufdtd), ("output_kufdtd", output_kufdtd),
         ("cpml_kappa_kufdtd", cpml_kappa_kufdtd))


def main():
    if not build_ref.build():
        raise SystemExit("reference checkout or x86_64 host not available")
    # one generator per case, seeded by its position, so a case can be
    # regenerated alone (python make_golden.py drude_kufdtd) without touching the others;
    # the first four keep the single shared stream they were made with
    only = set(sys.argv[1:])
    rng = np.random.default_rng(20261203)
    for pos, (name, fn) in enumerate(CASES):
        if pos >= 4:
            rng = np.random.default_rng(20261203 + pos)
        data = fn(rng)
        if only and name not in only:
            continue
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()

"""ctypes front end of the C oracle (test infrastructure only).

Every function mirrors one reference routine (file:line citations live in
fdtd_oracle.c) and works in place on NumPy arrays of logical shape
(nx, ny, nz); float32 arrays run the FP32 build, float64 arrays the FP64
build.  Arrays may be z-padded views (z stride 1, larger y/x strides).
"""
import ctypes as C
import math

import numpy as np

from . import build as _build

__all__ = ["update_e", "update_h", "pbc_e", "pbc_h", "cpml_e", "cpml_h",
           "add_points", "symp_h", "symp_e", "cpml_tables", "pulse",
           "OracleSim", "lib", "symp_h_scalar", "symp_cpml_e", "symp_cpml_h", "symp_stage_tables",
           "drude_e", "drude_coefficients"]

_LIBS = {}


def lib(kind):
    if kind not in _LIBS:
        _build.build()
        _LIBS[kind] = C.CDLL(_build.lib_path(kind))
    return _LIBS[kind]


def _kind(a):
    if a.dtype == np.float32:
        return "f32", C.c_float
    if a.dtype == np.float64:
        return "f64", C.c_double
    raise TypeError("oracle arrays must be float32 or float64, got %s" % a.dtype)


def _grid(a):
    if a.ndim != 3 or a.strides[2] != a.itemsize:
        raise ValueError("oracle arrays must be 3-D with unit z stride")
    it = a.itemsize
    return (C.c_int64 * 5)(a.shape[0], a.shape[1], a.shape[2],
                           a.strides[0] // it, a.strides[1] // it)


def _p(a):
    if a is None:
        return None
    return C.c_void_p(a.ctypes.data)


def _check(ref, *arrs):
    for a in arrs:
        if a is None:
            continue
        if a.dtype != ref.dtype or a.shape != ref.shape or a.strides != ref.strides:
            raise ValueError("oracle arrays must share dtype, shape and strides")


def update_e(ex, ey, ez, hx, hy, hz, cex, cey, cez):
    _check(ex, ey, ez, hx, hy, hz, cex, cey, cez)
    k, _ = _kind(ex)
    getattr(lib(k), "orc_update_e_" + k)(_grid(ex), *map(_p, (ex, ey, ez, hx, hy, hz, cex, cey, cez)))


def update_h(ex, ey, ez, hx, hy, hz, chx=None, chy=None, chz=None):
    _check(ex, ey, ez, hx, hy, hz, chx, chy, chz)
    k, _ = _kind(ex)
    getattr(lib(k), "orc_update_h_" + k)(_grid(ex), *map(_p, (ex, ey, ez, hx, hy, hz, chx, chy, chz)))


def pbc_e(axes, ex, ey, ez):
    k, _ = _kind(ex)
    getattr(lib(k), "orc_pbc_e_" + k)(_grid(ex), C.c_int(axes), _p(ex), _p(ey), _p(ez))


def pbc_h(axes, hx, hy, hz):
    k, _ = _kind(hx)
    getattr(lib(k), "orc_pbc_h_" + k)(_grid(hx), C.c_int(axes), _p(hx), _p(hy), _p(hz))


def _tables(t, key, dtype):
    arrs = [np.ascontiguousarray(t[key][a], dtype=dtype) if t[key][a] is not None and len(t[key][a])
            else np.zeros(1, dtype) for a in range(3)]
    ptrs = (C.c_void_p * 3)(*[a.ctypes.data for a in arrs])
    return arrs, ptrs


def _cpml(fn, npml, faces, tables, which, f_upd, f_src, coef, psi):
    """Common driver: which = 'e' or 'h'."""
    ref = f_upd[0]
    k, _ = _kind(ref)
    keep = []
    ptrs = []
    for name in ("b", "a", "km1"):
        arrs, p = _tables(tables, name + "_" + which, ref.dtype)
        keep.append(arrs)
        ptrs.append(p)
    psi_p = (C.c_void_p * 6)(*[(p.ctypes.data if p is not None else 0) for p in psi])
    npml_c = (C.c_int32 * 3)(*npml)
    getattr(lib(k), fn + k)(_grid(ref), npml_c, C.c_int(faces), ptrs[0], ptrs[1], ptrs[2],
                            *map(_p, f_upd if which == "e" else f_src),
                            *map(_p, f_src if which == "e" else f_upd),
                            *map(_p, coef), psi_p)


def cpml_e(npml, faces, tables, ex, ey, ez, hx, hy, hz, cex, cey, cez, psi_e):
    """psi_e = [eyx, ezx, ezy, exy, exz, eyz] (None where an axis has no PML)."""
    _cpml("orc_cpml_e_", npml, faces, tables, "e", (ex, ey, ez), (hx, hy, hz), (cex, cey, cez), psi_e)


def cpml_h(npml, faces, tables, ex, ey, ez, hx, hy, hz, psi_h, chx=None, chy=None, chz=None):
    """psi_h = [hyx, hzx, hzy, hxy, hxz, hyz]."""
    _cpml("orc_cpml_h_", npml, faces, tables, "h", (hx, hy, hz), (ex, ey, ez), (chx, chy, chz), psi_h)


def add_points(f, offsets, amps):
    k, _ = _kind(f)
    offsets = np.ascontiguousarray(offsets, np.int64)
    amps = np.ascontiguousarray(amps, f.dtype)
    getattr(lib(k), "orc_add_points_" + k)(_p(f), _p(offsets), _p(amps), C.c_int64(len(offsets)))


def symp_h(cl, ex, ey, ez, hx, hy, hz, chx, chy, chz):
    _check(ex, ey, ez, hx, hy, hz, chx, chy, chz)
    k, ct = _kind(ex)
    getattr(lib(k), "orc_symp_h_" + k)(_grid(ex), ct(cl), *map(_p, (ex, ey, ez, hx, hy, hz, chx, chy, chz)))


def symp_e(dl, ex, ey, ez, hx, hy, hz, cex, cey, cez):
    _check(ex, ey, ez, hx, hy, hz, cex, cey, cez)
    k, ct = _kind(ex)
    getattr(lib(k), "orc_symp_e_" + k)(_grid(ex), ct(dl), *map(_p, (ex, ey, ez, hx, hy, hz, cex, cey, cez)))


# --------------------------------------------------------------------------
# Coefficient formulas, restated independently of the product's host code.
# kappa/sigma/b/a: kuFDTD/before_CUDA/v0.3.0/boundary/cpml.py:126-136
# alpha grading:   KEMP/v0.7_pml/fdtd3d/naive/pml.py:35-36
# sigma_max from the target reflection R (normalised units, eta0 = 1).
# --------------------------------------------------------------------------
def cpml_tables(npml, m=4, R=1e-8, kappa_max=5.0, alpha_max=0.05, m_alpha=1, dt=0.5):
    """FP64 tables for one axis: dict with b_e, a_e, km1_e, b_h, a_h, km1_h (2P each)."""
    P = int(npml)
    out = {}
    if P == 0:
        return {k: np.zeros(0) for k in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}
    sigma_max = -(m + 1) * math.log(R) / (2.0 * P)
    depth_e = [P - s - 0.5 for s in range(P)] + [s + 0.5 for s in range(P)]
    depth_h = [float(P - s) for s in range(P)] + [float(s + 1) for s in range(P)]
    for tag, depth in (("e", depth_e), ("h", depth_h)):
        b, a, km1 = [], [], []
        for d in depth:
            x = d / P
            sig = sigma_max * x ** m
            kap = 1.0 + (kappa_max - 1.0) * x ** m
            alp = alpha_max * (1.0 - x) ** m_alpha
            bb = math.exp(-(sig / kap + alp) * dt)
            den = sig * kap + alp * kap * kap
            aa = sig / den * (bb - 1.0) if den > 0 else 0.0
            b.append(bb)
            a.append(aa)
            km1.append(1.0 / kap - 1.0)
        out["b_" + tag] = np.array(b)
        out["a_" + tag] = np.array(a)
        out["km1_" + tag] = np.array(km1)
    return out


def pulse(n, t0=150.0, width=30.0, freq=0.05):
    """Gaussian-modulated sine at integer step n (FP64):
    sin(2*pi*freq*n) * exp(-0.5*((n - t0)/width)**2)
    (2nd_order-Yee/Numpy/new_pml_test/gaussian.py:7-8,27)."""
    return math.sin(2.0 * math.pi * freq * n) * math.exp(-0.5 * ((n - t0) / width) ** 2)


def drude_e(box, ex, ey, ez, cex, cey, cez, J, CJA, CJB):
    """Drude ADE on the sub-box box = (i0, j0, k0) of the E arrays
    (kuFDTD drude_ade.c update_e); J, CJA, CJB: 3 dense arrays each, shape
    (ni, nj, nk), of the E arrays' dtype.  J is updated in place."""
    _check(ex, ey, ez, cex, cey, cez)
    kind, _ = _kind(ex)
    ni, nj, nk = J[0].shape
    for a in (*J, *CJA, *CJB):
        if a.dtype != ex.dtype or a.shape != (ni, nj, nk) or not a.flags.c_contiguous:
            raise ValueError("J, CJA, CJB must be C-contiguous (ni, nj, nk) arrays of the field dtype")
    i0, j0, k0 = (int(v) for v in box)
    if i0 < 0 or j0 < 0 or k0 < 0 or i0 + ni > ex.shape[0] or j0 + nj > ex.shape[1] or k0 + nk > ex.shape[2]:
        raise ValueError("Drude box outside the grid")
    b = (C.c_int64 * 6)(i0, j0, k0, ni, nj, nk)
    getattr(lib(kind), "orc_drude_e_" + kind)(_grid(ex), b, *map(_p, (ex, ey, ez, cex, cey, cez)),
                                              *map(_p, J), *map(_p, CJA), *map(_p, CJB))


def drude_coefficients(pfreq, gamma, dt=0.5):
    """CJA = (2 - gamma dt)/(2 + gamma dt), CJB = 4 (dt pfreq)^2/(2 + gamma dt), in
    float32 array arithmetic as kuFDTD/v0.2.0/dim3/cpu/matter.py:198-208 (and
    268-278) evaluates them on its 'f' arrays."""
    g = np.asarray(gamma, np.float32)
    w = np.asarray(pfreq, np.float32)
    g, w = np.broadcast_arrays(g, w)
    dt32 = np.float32(dt)
    tmp = np.float32(2) + g * dt32
    cja = (np.float32(2) - g * dt32) / tmp
    cjb = np.float32(4) * (dt32 * w) ** 2 / tmp
    return cja.astype(np.float32), cjb.astype(np.float32)


class OracleSim:
    """Whole-step oracle: state in NumPy arrays, canonical step order.

    fields: dict ex..hz, cex..cez (+ optional chx..chz), all of one dtype.
    npml: (Px, Py, Pz); faces bitmask; tables: per-axis dicts from
    cpml_tables merged as tables[name][axis].
    sources: list of (component, (i, j, k), amplitude-table) where the
    amplitude table is indexed by the 1-based step number.
    """

    def __init__(self, fields, npml=(0, 0, 0), faces=0x3F, tables=None, sources=(), drude=None):
        # drude: optional (box (i0, j0, k0), J[3], CJA[3], CJB[3]) applied after update_e
        # (kuFDTD/v0.2.0/dim3/cpu/test/030-drude-cpml.py:88-92 step order)
        self.drude = drude
        self.f = fields
        ex = fields["ex"]
        self.dtype = ex.dtype
        nx, ny, nz = ex.shape
        self.npml = tuple(int(p) for p in npml)
        self.faces = faces
        self.tables = tables
        self.sources = list(sources)
        self.tstep = 1
        shapes = [(2 * self.npml[0], ny, nz), (nx, 2 * self.npml[1], nz), (nx, ny, 2 * self.npml[2])]
        self.psi_e = []
        self.psi_h = []
        for ax in range(3):
            for _ in range(2):
                self.psi_e.append(np.zeros(shapes[ax], self.dtype) if self.npml[ax] else None)
                self.psi_h.append(np.zeros(shapes[ax], self.dtype) if self.npml[ax] else None)

    def step(self, n=1):
        f = self.f
        E = (f["ex"], f["ey"], f["ez"])
        H = (f["hx"], f["hy"], f["hz"])
        CE = (f["cex"], f["cey"], f["cez"])
        CH = (f.get("chx"), f.get("chy"), f.get("chz"))
        pml = any(self.npml)
        for _ in range(n):
            update_e(*E, *H, *CE)
            if self.drude is not None:
                box, J, CJA, CJB = self.drude
                drude_e(box, *E, *CE, J, CJA, CJB)
            if pml:
                cpml_e(self.npml, self.faces, self.tables, *E, *H, *CE, self.psi_e)
            for comp, (i, j, k), amp in self.sources:
                arr = f[comp]
                arr[i, j, k] = arr[i, j, k] + np.asarray(amp[self.tstep], dtype=self.dtype)
            update_h(*E, *H, *CH)
            if pml:
                cpml_h(self.npml, self.faces, self.tables, *E, *H, self.psi_h, *CH)
            self.tstep += 1


def symp_h_scalar(cl, ch, ex, ey, ez, hx, hy, hz):
    _check(ex, ey, ez, hx, hy, hz)
    k, ct = _kind(ex)
    getattr(lib(k), "orc_symp_h_scalar_" + k)(_grid(ex), ct(cl), ct(ch), *map(_p, (ex, ey, ez, hx, hy, hz)))


def _symp_cpml(fn, npml, faces, coef_args, tables, which, E, H, coef, psi):
    ref = E[0]
    k, ct = _kind(ref)
    keep, ptrs = [], []
    for name in ("b", "a", "km1"):
        arrs, pp = _tables(tables, name + "_" + which, ref.dtype)
        keep.append(arrs)
        ptrs.append(pp)
    psi_p = (C.c_void_p * 6)(*[(p.ctypes.data if p is not None else 0) for p in psi])
    npml_c = (C.c_int32 * 3)(*npml)
    getattr(lib(k), fn + k)(_grid(ref), npml_c, C.c_int(faces), *[ct(v) for v in coef_args],
                            ptrs[0], ptrs[1], ptrs[2], *map(_p, E), *map(_p, H), *map(_p, coef), psi_p)


def symp_cpml_e(npml, faces, dl, tables, ex, ey, ez, hx, hy, hz, cex, cey, cez, psi_e):
    """4th-order CPML E-stage correction; tables: stage tables (b_e, a_e, km1_e per axis)."""
    _symp_cpml("orc_symp_cpml_e_", npml, faces, (dl,), tables, "e", (ex, ey, ez), (hx, hy, hz),
               (cex, cey, cez), psi_e)


def symp_cpml_h(npml, faces, cl, ch_scalar, tables, ex, ey, ez, hx, hy, hz, psi_h, chx=None, chy=None, chz=None):
    _symp_cpml("orc_symp_cpml_h_", npml, faces, (cl, ch_scalar), tables, "h", (ex, ey, ez), (hx, hy, hz),
               (chx, chy, chz), psi_h)


def symp_stage_tables(npml, coef, S=0.743, m=4, R=1e-8, kappa_max=5.0, alpha_max=0.05, m_alpha=1):
    """Stage tables of the 4th-order CPML: cpml_tables with the sub-step coef*S."""
    return cpml_tables(npml, m=m, R=R, kappa_max=kappa_max, alpha_max=alpha_max, m_alpha=m_alpha, dt=coef * S)

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
           "drude_e", "drude_coefficients", "TfsfNormal", "output_data"]

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


class TfsfNormal:
    """Total-field/scattered-field plane wave at normal incidence, restated from
    kuFDTD/v0.2.0/dim3/tfsf.py (test infrastructure only).

    pt1, pt2: corners of the total-field box as Tfsf.set_space receives them
    (None -> 1 / n-2), faces: 6 flags (x front, x back, y front, ... as
    apply_direction 'fb'), axis 0..2: propagation axis, angle: polarisation
    angle, wdt: wfreq*dt (the source phase step).  Arrays are float32; NumPy
    1.x casting as in 2009 (scalar coefficients taken to float32).

      Fdtd1d                 tfsf.py:14-40 (E, H of N+10 cells, Mur-like
                             two-step delay at both ends, hard source E[3])
      faces                  tfsf.py:140-186 (calc_face_list)
      incident coefficients  tfsf.py:189-231 (calc_inc_list)
      updateE / updateH      tfsf.py:234-244, TfsfFace tfsf.py:68-89
    """

    def __init__(self, shape, pt1, pt2, faces, axis, angle, wdt):
        n3 = list(shape)
        p1 = [1 if v is None else int(v) for v in pt1]
        p2 = [n3[a] - 2 if v is None else int(v) for a, v in enumerate(pt2)]
        p2 = [v + 1 for v in p2]
        self.p1, self.p2, self.axis, self.faces = p1, p2, int(axis), [bool(f) for f in faces]
        N = p2[axis] - p1[axis] + 1
        self.E = np.zeros(N + 10, np.float32)
        self.H = np.zeros(N + 10, np.float32)
        self.abc = [np.float32(0)] * 4   # f1, f2, b1, b2
        self.wdt = float(wdt)
        si, co = np.float32(math.sin(angle)), np.float32(math.cos(angle))
        # (ce1, ce2, ch1, ch2, sE1, sE2, sH1, sH2) of Inc1..Inc6; slice ids 1..5 of tfsf.py:195-199
        zero = np.float32(0)
        self.incs = [(-si, co, co, si, 1, 1, 2, 2), (si, -co, -co, -si, 5, 5, 5, 5),
                     (zero, si, zero, -co, 4, 3, 3, 4), (zero, -si, zero, co, 4, 3, 3, 4),
                     (-co, zero, -si, zero, 3, 4, 4, 3), (co, zero, si, zero, 3, 4, 4, 3)]
        order = {0: [0, 1, 2, 3, 4, 5], 1: [4, 5, 0, 1, 2, 3], 2: [2, 3, 4, 5, 0, 1]}[self.axis]
        self.face_inc = order   # face f (xf, xb, yf, yb, zf, zb) uses Inc order[f]

    def _sl1d(self, sid):
        i1, i2 = 5, self.p2[self.axis] - self.p1[self.axis] + 5
        return {1: slice(i1 - 1, i1), 2: slice(i1, i1 + 1), 3: slice(i1, i2), 4: slice(i1, i2 + 1),
                5: slice(i2, i2 + 1)}[sid]

    def update_e1d(self, tstep):
        E, H = self.E, self.H
        E[1:-1] -= np.float32(0.5) * (H[2:] - H[1:-1])
        E[0] = self.abc[0]
        self.abc[0] = self.abc[1]
        self.abc[1] = E[1]
        E[-1] = self.abc[2]
        self.abc[2] = self.abc[3]
        self.abc[3] = E[-2]
        E[3] = np.float32(math.sin(self.wdt * tstep))

    def update_h1d(self):
        self.H[1:] -= np.float32(0.5) * (self.E[1:] - self.E[:-1])

    def _faces(self, f):
        """(e1, e2, h1, h2) component names and their index tuples (tfsf.py:140-186)."""
        (i1, j1, k1), (i2, j2, k2) = self.p1, self.p2
        sx, sxp, sy, syp, sz, szp = (slice(i1, i2), slice(i1, i2 + 1), slice(j1, j2), slice(j1, j2 + 1),
                                      slice(k1, k2), slice(k1, k2 + 1))
        return [
            (("ey", "ez", "hy", "hz"), ((i1 - 1, syp, sz), (i1 - 1, sy, szp), (i1, sy, szp), (i1, syp, sz))),
            (("ey", "ez", "hy", "hz"), ((i2, syp, sz), (i2, sy, szp), (i2, sy, szp), (i2, syp, sz))),
            (("ez", "ex", "hz", "hx"), ((sx, j1 - 1, szp), (sxp, j1 - 1, sz), (sxp, j1, sz), (sx, j1, szp))),
            (("ez", "ex", "hz", "hx"), ((sx, j2, szp), (sxp, j2, sz), (sxp, j2, sz), (sx, j2, szp))),
            (("ex", "ey", "hx", "hy"), ((sxp, sy, k1 - 1), (sx, syp, k1 - 1), (sx, syp, k1), (sxp, sy, k1))),
            (("ex", "ey", "hx", "hy"), ((sxp, sy, k2), (sx, syp, k2), (sx, syp, k2), (sxp, sy, k2))),
        ][f]

    def _inc(self, f, eh):
        """The two incident arrays of face f for E (eh=0: the face's E update reads
        the 1-D H) or H (eh=1), broadcast to the face slices (newaxis of tfsf.py:201-214)."""
        ce1, ce2, ch1, ch2, sE1, sE2, sH1, sH2 = self.incs[self.face_inc[f]]
        if eh == 0:
            c1, c2, a1, a2 = ch1, ch2, self.H[self._sl1d(sH1)], self.H[self._sl1d(sH2)]
        else:
            c1, c2, a1, a2 = ce1, ce2, self.E[self._sl1d(sE1)], self.E[self._sl1d(sE2)]
        newaxis = {0: [0, 0, 1, 1, 1, 1], 1: [1, 1, 0, 0, 0, 0], 2: [0, 0, 0, 0, 0, 0]}[self.axis][f]
        ex = [slice(None)]
        ex.insert(newaxis, None)
        return (c1 * a1)[tuple(ex)], (c2 * a2)[tuple(ex)]

    def update_e(self, fields, tstep):
        """tfsf.py:234-237: 1-D E step, then E += 0.5 * incident H on every face."""
        self.update_e1d(tstep)
        for f in range(6):
            if not self.faces[f]:
                continue
            names, idx = self._faces(f)
            h1, h2 = self._inc(f, 0)
            fields[names[0]][idx[0]] += np.float32(0.5) * h1
            fields[names[1]][idx[1]] += np.float32(0.5) * h2

    def update_h(self, fields):
        """tfsf.py:240-244: 1-D H step, then H += 0.5 * incident E on every face."""
        self.update_h1d()
        for f in range(6):
            if not self.faces[f]:
                continue
            names, idx = self._faces(f)
            e1, e2 = self._inc(f, 1)
            fields[names[2]][idx[2]] += np.float32(0.5) * e1
            fields[names[3]][idx[3]] += np.float32(0.5) * e2


def output_data(fields, dataform, pt1, pt2, step=(1, 1, 1)):
    """kuFDTD Output.get_data() restated in NumPy (kuFDTD/v0.2.0/dim3/output.py:
    set_space 33-46, centred data 167-178, square/sum/sqrt 181-195, Poynting
    198-211); fields: dict ex..hz of float32 (nx, ny, nz) arrays."""
    d = dataform.lower()
    n = fields["ex"].shape
    p1 = [1 if v is None else int(v) for v in pt1]
    p2 = [n[a] - 2 if v is None else int(v) for a, v in enumerate(pt2)]
    (i1, j1, k1), (i2, j2, k2) = p1, p2
    sl = (slice(i1, i2 + 1), slice(j1, j2 + 1), slice(k1, k2 + 1))
    up = lambda a: tuple(slice(x.start + 1, x.stop + 1) if q == a else x for q, x in enumerate(sl))
    up2 = lambda a, b: tuple(slice(x.start + 1, x.stop + 1) if q in (a, b) else x for q, x in enumerate(sl))
    st = tuple(slice(None, None, int(v)) for v in step)
    def ce(q):
        E = fields["e" + "xyz"[q]]
        return (0.5 * (E[sl] + E[up(q)]))[st]
    def ch(q):
        H = fields["h" + "xyz"[q]]
        a, b = [(1, 2), (0, 2), (0, 1)][q]
        return (0.25 * (H[sl] + H[up(a)] + H[up(b)] + H[up2(a, b)]))[st]
    if d[0] in "eh":
        cen = ce if d[0] == "e" else ch
        if len(d) >= 2 and d[1] in "xyz":
            v = cen("xyz".index(d[1]))
            out = v ** 2 if d.endswith("2") and len(d) == 3 else v
        else:
            tot = 0
            for q in range(3):
                tot = tot + cen(q) ** 2
            out = np.sqrt(tot) if len(d) == 1 else tot
    else:
        ex, ey, ez, hx, hy, hz = ce(0), ce(1), ce(2), ch(0), ch(1), ch(2)
        S = [ey * hz - ez * hy, ez * hx - ex * hz, ex * hy - ey * hx]
        if len(d) >= 2 and d[1] in "xyz":
            v = S["xyz".index(d[1])]
            out = v ** 2 if len(d) == 3 else v
        else:
            tot = 0
            for q in range(3):
                tot = tot + S[q] ** 2
            out = np.sqrt(tot) if len(d) == 1 else tot
    ds = tuple(0 if p2[a] == p1[a] else slice(None) for a in range(3))
    return out[ds]


class OracleSim:
    """Whole-step oracle: state in NumPy arrays, canonical step order.

    fields: dict ex..hz, cex..cez (+ optional chx..chz), all of one dtype.
    npml: (Px, Py, Pz); faces bitmask; tables: per-axis dicts from
    cpml_tables merged as tables[name][axis].
    sources: list of (component, (i, j, k), amplitude-table) where the
    amplitude table is indexed by the 1-based step number.
    """

    def __init__(self, fields, npml=(0, 0, 0), faces=0x3F, tables=None, sources=(), drude=None, tfsf=None):
        # drude: optional (box (i0, j0, k0), J[3], CJA[3], CJB[3]) applied after update_e
        # (kuFDTD/v0.2.0/dim3/cpu/test/030-drude-cpml.py:88-92 step order);
        # tfsf: optional TfsfNormal applied after cpml_e and after cpml_h
        # (kuFDTD/v0.2.0/dim3/cpu/test/200-dielectric-cpml-output-tfsf.py:72-78), point sources after it
        self.drude = drude
        self.tfsf = tfsf
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
            if self.tfsf is not None:
                self.tfsf.update_e(f, self.tstep)
            for comp, (i, j, k), amp in self.sources:
                arr = f[comp]
                arr[i, j, k] = arr[i, j, k] + np.asarray(amp[self.tstep], dtype=self.dtype)
            update_h(*E, *H, *CH)
            if pml:
                cpml_h(self.npml, self.faces, self.tables, *E, *H, self.psi_h, *CH)
            if self.tfsf is not None:
                self.tfsf.update_h(f)
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

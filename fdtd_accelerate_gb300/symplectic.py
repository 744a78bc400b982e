"""4th-order spatial / 4-stage symplectic FDTD on CUDA float32 tensors.

Reference: 4th_order-Symplectic/PyCUDA/100-base.py (kernels :10-44, integrator
:58-63 and :124-141) and 4th_order-Symplectic/Python-C/dielectric.c:5-96.
One step is

    for sn in 0..3:  H stage (cl[sn]);  E stage (dl[sn]);  sources at t = tn + sn/5
    H stage (cl[4])

with cl = [c1, c2, c3, c2, c1], dl = [d1, d2, d2, d1, 0] (the closing H stage
uses cl[4]; the C driver's cl[sn] at Python-C/100-base.py:69-72 is not
followed).  Coefficients ce = (S/24)/eps_r, ch = S/24, S = 0.743
(Python-C/100-base.py:11,28).

CPML: the reference has none for this scheme; here each stage applies the
kappa CPML of the 2nd-order scheme with the stage's sub-step: b = exp(-(sigma/
kappa + alpha) * c * S), a = sigma/(sigma kappa + alpha kappa^2) (b - 1), and the
stage stencil's 4th-order derivative (fdtd_symplectic_cpml_{e,h}_f32).
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _native as N
from .api import check_field_tensors, grid_of, stream_of
from .cpml import parse_faces, sigma_max_from_reflection
from .sources import PointSources

__all__ = ["C1", "C2", "C3", "D1", "D2", "CL", "DL", "COURANT", "update_h", "update_e",
           "stage_tables", "SymplecticCpml", "SymplecticSolver"]

C1, C2, C3 = 0.17399689146541, -0.12038504121430, 0.89277629949778
D1, D2 = 0.62337932451322, -0.12337932451322
CL = (C1, C2, C3, C2, C1)
DL = (D1, D2, D2, D1, 0.0)
COURANT = 0.743


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _check_dims(nx, ny, nz, ref):
    if (nx, ny, nz) != tuple(ref.shape):
        raise ValueError("nx, ny, nz = %s do not match the arrays %s" % ((nx, ny, nz), tuple(ref.shape)))


def update_h(nx, ny, nz, cl, ex, ey, ez, hx, hy, hz, chx, chy=None, chz=None):
    """H stage, signature of dielectric.update_h (Python-C/dielectric.c:5-14).
    chx may be a float (uniform ch) with chy = chz = None."""
    names = ["ex", "ey", "ez", "hx", "hy", "hz"]
    ts = [ex, ey, ez, hx, hy, hz]
    scalar = isinstance(chx, (int, float))
    if not scalar:
        names += ["chx", "chy", "chz"]
        ts += [chx, chy, chz]
    ref = check_field_tensors(names, ts)
    _check_dims(nx, ny, nz, ref)
    g = grid_of(ref)
    with torch.cuda.device(ref.device):
        if scalar:
            N.call("fdtd_symplectic_h_scalar_f32", C.byref(g), float(cl), float(chx),
                   *map(_p, (ex, ey, ez, hx, hy, hz)), stream_of(ref))
        else:
            N.call("fdtd_symplectic_h_f32", C.byref(g), float(cl), *map(_p, ts), stream_of(ref))


def update_e(nx, ny, nz, dl, ex, ey, ez, hx, hy, hz, cex, cey, cez):
    """E stage, signature of dielectric.update_e (Python-C/dielectric.c:52-61)."""
    ts = (ex, ey, ez, hx, hy, hz, cex, cey, cez)
    ref = check_field_tensors(("ex", "ey", "ez", "hx", "hy", "hz", "cex", "cey", "cez"), ts)
    _check_dims(nx, ny, nz, ref)
    g = grid_of(ref)
    with torch.cuda.device(ref.device):
        N.call("fdtd_symplectic_e_f32", C.byref(g), float(dl), *map(_p, ts), stream_of(ref))


def stage_tables(npml, coef, S=COURANT, m=4, R=1e-8, kappa_max=5.0, alpha_max=0.05, m_alpha=1):
    """FP64 CPML tables of one stage (sub-step coef*S): b_e, a_e, b_h, a_h, km1_e, km1_h."""
    P = int(npml)
    smax = sigma_max_from_reflection(P, m, R)
    s = np.arange(P, dtype=np.float64)
    out = {}
    for tag, d in (("e", np.concatenate([P - s - 0.5, s + 0.5])), ("h", np.concatenate([P - s, s + 1.0]))):
        x = d / P
        sig = smax * x ** m
        kap = 1.0 + (kappa_max - 1.0) * x ** m
        alp = alpha_max * (1.0 - x) ** m_alpha
        b = np.exp(-(sig / kap + alp) * (coef * S))
        den = sig * kap + alp * kap * kap
        out["b_" + tag] = b
        out["a_" + tag] = np.where(den > 0, sig / np.where(den > 0, den, 1.0) * (b - 1.0), 0.0)
        out["km1_" + tag] = 1.0 / kap - 1.0
    return out


class SymplecticCpml:
    """Device tables for every distinct stage coefficient and psi slabs."""

    def __init__(self, shape, npml, faces=0x3F, S=COURANT, device="cuda", **params):
        nx, ny, nz = shape
        if isinstance(npml, int):
            npml = (npml,) * 3
        faces = parse_faces(faces)
        npml = [int(p) if (faces >> (2 * a)) & 3 else 0 for a, p in enumerate(npml)]
        for a, (p, n) in enumerate(zip(npml, shape)):
            if p and n < 2 * p + 2:
                raise ValueError("axis %d: %d CPML cells need at least %d cells" % (a, p, 2 * p + 2))
        self.npml, self.faces, self.S = tuple(npml), faces, S
        self.device = torch.device(device)
        f32 = lambda v: torch.tensor(v, dtype=torch.float32, device=self.device)
        self.tables = {}
        for coef in sorted(set(CL) | set(DL[:4])):
            t = [stage_tables(p, coef, S, **params) if p else None for p in npml]
            self.tables[coef] = [{k: f32(v) for k, v in ta.items()} if ta else None for ta in t]
        pshapes = [(2 * npml[0], ny, nz), (nx, 2 * npml[1], nz), (nx, ny, 2 * npml[2])]
        z = lambda a: torch.zeros(pshapes[a], dtype=torch.float32, device=self.device) if npml[a] else None
        self._pshapes = pshapes
        self.psi_e = [z(a) for a in range(3) for _ in range(2)]
        # H psi of the current state buffer; the fused stage-pair path keeps a
        # second set (hbuf[1 - hcur]) that it writes while it reads this one
        self.hbuf = [[z(a) for a in range(3) for _ in range(2)], None]
        self.hcur = 0
        self._structs = {c: self._make_struct(c) for c in self.tables}
        self._psi = N.Psi()
        self._fill_psi()

    @property
    def psi_h(self):
        return self.hbuf[self.hcur]

    def _fill_psi(self):
        for q in range(6):
            self._psi.e[q] = self.psi_e[q].data_ptr() if self.psi_e[q] is not None else None
            self._psi.h[q] = self.psi_h[q].data_ptr() if self.psi_h[q] is not None else None

    def second_h_buffer(self):
        """Allocate the second H psi set (stage-pair path) and return both."""
        if self.hbuf[1] is None:
            self.hbuf[1] = [torch.zeros_like(t) if t is not None else None for t in self.hbuf[0]]
        return self.hbuf

    def set_hcur(self, b):
        if b != self.hcur:
            self.hcur = b
            self._fill_psi()

    @property
    def active(self):
        return any(self.npml)

    def _make_struct(self, coef):
        c = N.Cpml()
        for a in range(3):
            c.npml[a] = self.npml[a]
        c.faces = self.faces
        for a in range(3):
            t = self.tables[coef][a]
            for key in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h"):
                getattr(c, key)[a] = t[key].data_ptr() if t else None
        return c

    def update_h(self, cl, ch, f, stream):
        """f = (ex, ey, ez, hx, hy, hz); ch a float or three arrays."""
        g = grid_of(f[0])
        chs = (None, None, None) if isinstance(ch, (int, float)) else ch
        chv = float(ch) if isinstance(ch, (int, float)) else 0.0
        N.call("fdtd_symplectic_cpml_h_f32", C.byref(g), C.byref(self._structs[cl]), float(cl), chv,
               *map(_p, f), *map(_p, chs), C.byref(self._psi), stream)

    def update_e(self, dl, f, ce, stream):
        """f = (ex, ey, ez, hx, hy, hz); ce three arrays."""
        g = grid_of(f[0])
        N.call("fdtd_symplectic_cpml_e_f32", C.byref(g), C.byref(self._structs[dl]), float(dl),
               *map(_p, f), *map(_p, ce), C.byref(self._psi), stream)


class SymplecticSolver:
    """4-stage symplectic 4th-order FDTD on one GPU.

    ce: three eps-weighted E coefficient arrays ((S/24)/eps_r); ch: a float
    (uniform, default S/24) or three arrays; sources: (component, (i, j, k),
    amplitude) with amplitude a callable of continuous time t (FP64), added
    after every E stage at t = tn + sn/5 (PyCUDA/100-base.py:136).
    fused: take the stage-pair path (one pass per H + E stage pair: the pair
    kernel inside, the edge kernels on the y/z CPML shell) where pair_path()
    allows; bit-identical to the per-stage kernels and faster than them
    (8.25 against 12.3 ms per step on the 512^3 workload); fused=False keeps
    the one-launch-per-stage path.  x_chunk: x planes per work item of the
    pair kernel (0: chosen per tiling by the plan).
    """

    def __init__(self, shape, ce=None, ch=None, npml=0, faces=0x3F, sources=(), device="cuda",
                 S=COURANT, cpml_params=None, max_steps=0, fused=True, x_chunk=0):
        self.shape = tuple(int(v) for v in shape)
        self.device = torch.device(device)
        dev = self.device
        self.S = S
        # state buffers: buf[cur] holds the fields; the stage-pair path writes
        # buf[1 - cur] from buf[cur] (the second buffer is allocated on first use)
        self._buf = [torch.zeros((6,) + self.shape, dtype=torch.float32, device=dev), None]
        self._cur = 0
        self.fused = fused
        self.x_chunk = int(x_chunk)
        self._pair = None
        self._pair_src = None
        if ce is None:
            ce = [np.full(self.shape, S / 24.0)] * 3
        self.ce = [torch.as_tensor(c, dtype=torch.float32, device=dev).contiguous() for c in ce]
        self.ch = float(S / 24.0) if ch is None else (
            float(ch) if isinstance(ch, (int, float)) else
            [torch.as_tensor(c, dtype=torch.float32, device=dev).contiguous() for c in ch])
        self.cpml = SymplecticCpml(self.shape, npml, faces, S, device=dev, **(cpml_params or {}))
        self.src_spec = list(sources)
        self.max_steps = max_steps
        self.tstep = 1
        self._src = None
        self._stage_args = None
        self._build_sources(max(max_steps, 1))

    def _build_sources(self, nsteps):
        tabs = []
        for comp, ijk, amp in self.src_spec:
            t = np.zeros(4 * (nsteps + 2), dtype=np.float64)
            for tn in range(1, nsteps + 2):
                for sn in range(4):
                    t[4 * tn + sn] = amp(tn + sn / 5.0)
            tabs.append((comp, ijk, t))
        self._src = PointSources(self.shape, tabs, device=self.device)
        self._src_steps = nsteps

    @property
    def f(self):
        """ex, ey, ez, hx, hy, hz of the current state buffer."""
        return list(self._buf[self._cur])

    @property
    def fields(self):
        return dict(zip(("ex", "ey", "ez", "hx", "hy", "hz"), self.f))

    def pair_path(self):
        """True when step() runs the fused stage pairs: uniform ch, rows of a
        multiple of 4 floats (16-byte TMA rows), fewer than 2^31 cells, every
        extent at least 4."""
        nx, ny, nz = self.shape
        return (self.fused and isinstance(self.ch, float) and nz % 4 == 0 and min(self.shape) >= 4
                and nx * ny * nz < 2 ** 31)

    def _pair_plan(self):
        if self._pair is not None and self._pair_src is self._src:
            return self._pair
        self.close()
        if self._buf[1] is None:
            self._buf[1] = torch.zeros_like(self._buf[0])
        hb = self.cpml.second_h_buffer()
        st = N.SympState()
        for b in range(2):
            for q in range(6):
                st.f[b][q] = self._buf[b][q].data_ptr()
                st.psi_h[b][q] = hb[b][q].data_ptr() if hb[b][q] is not None else None
        for q in range(6):
            e = self.cpml.psi_e[q]
            st.psi_e[q] = e.data_ptr() if e is not None else None
        for q in range(3):
            st.ce[q] = self.ce[q].data_ptr()
        if not hasattr(self, "_status"):
            self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        if not hasattr(self, "_queue"):
            self._queue = torch.zeros(2, dtype=torch.int32, device=self.device)
        h = C.c_void_p()
        src = self._src.struct()
        with torch.cuda.device(self.device):
            N.call("fdtd_symp_pair_plan_create", C.byref(h), C.byref(grid_of(self._buf[0][0])), C.byref(st),
                   C.byref(src), int(self.x_chunk), int(self._cur), C.c_void_p(self._status.data_ptr()),
                   C.c_void_p(self._queue.data_ptr()), stream_of(self._buf[0][0]))
        self._pair, self._pair_src = h, self._src
        return h

    def close(self):
        if self._pair is not None:
            N.lib().fdtd_symp_pair_plan_destroy(self._pair)
            self._pair = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check_status(self):
        """Raise if a bounded device wait of the stage-pair kernel expired."""
        if hasattr(self, "_status"):
            v = int(self._status.item())
            if v:
                self._status.zero_()
                N.check(v, "fdtd_symp_pair_run (device status)")

    def set_fields(self, **arrays):
        for k, v in arrays.items():
            self.fields[k].copy_(torch.as_tensor(v, dtype=torch.float32, device=self.device))

    def step(self, n=1):
        """Advance n steps.  On the stage-pair path (pair_path()): each H stage
        and the E stage after it run as one fused pass with the sources
        (fdtd_symp_pair_run), the closing H stage of a step merges with the
        opening H stage of the next into one pass, and the run's last H stage
        runs alone in place: 4 n passes and one H stage for n steps.  Otherwise
        step_stages()."""
        if n <= 0:
            return
        if not self.pair_path():
            return self.step_stages(n)
        if self.src_spec and self.tstep + n > self._src_steps:
            self._build_sources(self.tstep + n)
        plan = self._pair_plan()
        L = N.lib()
        L.fdtd_symp_pair_plan_set_current(plan, self._cur)
        cp = self.cpml
        tabs = (lambda c: C.byref(cp._structs[c])) if cp.active else (lambda c: None)
        ch = float(self.ch)
        with torch.cuda.device(self.device):
            stream = stream_of(self._buf[0][0])
            for m in range(n):
                tn = self.tstep + m
                for sn in range(4):
                    two = 1 if (sn == 0 and m > 0) else 0   # closing H(c1) of step tn-1, then H(c1)
                    cl_a = CL[4] if two else CL[sn]
                    N.call("fdtd_symp_pair_run", plan, tabs(cl_a), tabs(CL[sn]), tabs(DL[sn]), float(cl_a),
                           float(CL[sn]), two, float(DL[sn]), ch, 4 * tn + sn if self.src_spec else -1, stream)
                    self._cur = 1 - self._cur
                    cp.set_hcur(self._cur)
            self._stage_args = None
            self._fused_stage(0, CL[4], None, ch, stream)
        self.tstep += n

    def step_stages(self, n=1):
        """Advance n steps: one launch per stage (the stage update and its CPML
        slabs together, fdtd_symplectic_stage_f32) and the sources after each E
        stage.  Fields of 2^31 or more elements (the stage kernel's offsets are
        32-bit) take the per-call path of step_unfused."""
        f = self.f
        if f[0].numel() >= 2 ** 31:
            return self.step_unfused(n)
        if self.src_spec and self.tstep + n > self._src_steps:
            self._build_sources(self.tstep + n)
        self._stage_args = self._make_stage_args()
        g, fptr, ceptr, chptr, chv = self._stage_args
        with torch.cuda.device(self.device):
            stream = stream_of(f[0])
            for _ in range(n):
                tn = self.tstep
                for sn in range(4):
                    self._fused_stage(0, CL[sn], chptr, chv, stream)
                    self._fused_stage(1, DL[sn], ceptr, 0.0, stream)
                    if self.src_spec:
                        self._src.apply(4 * tn + sn, *f[:3])
                self._fused_stage(0, CL[4], chptr, chv, stream)
                self.tstep += 1

    def _make_stage_args(self):
        g = grid_of(self.f[0])
        fptr = (C.c_void_p * 6)(*(t.data_ptr() for t in self.f))
        ceptr = (C.c_void_p * 3)(*(t.data_ptr() for t in self.ce))
        if isinstance(self.ch, float):
            chptr, chv = None, self.ch
        else:
            chptr, chv = (C.c_void_p * 3)(*(t.data_ptr() for t in self.ch)), 0.0
        return g, fptr, ceptr, chptr, chv

    def _fused_stage(self, e_or_h, coef, cptr, chv, stream):
        if self._stage_args is None:
            self._stage_args = self._make_stage_args()
        g, fptr = self._stage_args[0], self._stage_args[1]
        cp = C.byref(self.cpml._structs[coef]) if self.cpml.active else None
        psi = C.byref(self.cpml._psi) if self.cpml.active else None
        N.call("fdtd_symplectic_stage_f32", C.byref(g), cp, int(e_or_h), float(coef), float(chv), fptr,
               cptr, psi, stream)

    def step_unfused(self, n=1):
        """The same steps through the reference-shaped calls: update_h /
        update_e per stage, then the per-axis CPML corrections."""
        nx, ny, nz = self.shape
        f, ce, ch = self.f, self.ce, self.ch
        if self.src_spec and self.tstep + n > self._src_steps:
            self._build_sources(self.tstep + n)
        with torch.cuda.device(self.device):
            stream = stream_of(f[0])
            for _ in range(n):
                tn = self.tstep
                for sn in range(4):
                    self._h_stage(CL[sn], stream)
                    update_e(nx, ny, nz, DL[sn], *f, *ce)
                    if self.cpml.active:
                        self.cpml.update_e(DL[sn], f, ce, stream)
                    if self.src_spec:
                        self._src.apply(4 * tn + sn, *f[:3])
                self._h_stage(CL[4], stream)
                self.tstep += 1

    def _h_stage(self, cl, stream):
        nx, ny, nz = self.shape
        f, ch = self.f, self.ch
        if isinstance(ch, float):
            update_h(nx, ny, nz, cl, *f, ch)
        else:
            update_h(nx, ny, nz, cl, *f, *ch)
        if self.cpml.active:
            self.cpml.update_h(cl, ch, f, stream)

"""FP64 runs on the GPU: the 2nd-order Yee step (fdtd_step_unfused_f64) and
the 4th-order symplectic stages (fdtd_symplectic_stage_f64).

The same step as YeeSolver (update_e, cpml_e, sources, update_h, cpml_h, in
the reference's operation order) evaluated in double precision.  The CPML
tables and source amplitudes are the FP32 values of the FP32 path widened to
double, so both paths solve the same discrete problem and their difference is
the FP32 rounding.  Used for accuracy checks at full size and for central
differences of a loss when checking the adjoint's gradient.
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N
from .cpml import CpmlLayer
from .sources import PointSources

__all__ = ["YeeRun64", "SympRun64", "family_errors"]

COMPONENTS6 = ("ex", "ey", "ez", "hx", "hy", "hz")


class YeeRun64:
    """shape, ce (3 arrays, any float dtype), npml, faces, cpml_params, sources
    as for YeeSolver; monitors: (component, (i, j, k)) with component ex..hz."""

    def __init__(self, shape, ce=None, npml=0, faces=0x3F, cpml_params=None, sources=(), monitors=(),
                 device="cuda"):
        nx, ny, nz = (int(v) for v in shape)
        self.shape = (nx, ny, nz)
        self.device = torch.device(device)
        dev = self.device
        self.f = torch.zeros((6, nx, ny, nz), dtype=torch.float64, device=dev)
        self.ce = torch.full((3, nx, ny, nz), 0.5, dtype=torch.float64, device=dev)
        if ce is not None:
            self.set_ce(ce)
        self.cpml = CpmlLayer(self.shape, npml, faces, device=dev, **(cpml_params or {}))
        self.psi_e = [torch.zeros_like(t, dtype=torch.float64) if t is not None else None
                      for t in self.cpml.psi_e[0]]
        self.psi_h = [torch.zeros_like(t, dtype=torch.float64) if t is not None else None for t in self.cpml.psi_h]
        self.sources = PointSources(self.shape, sources, device=dev)
        mons = list(monitors)
        for comp, ijk in mons:
            if comp not in COMPONENTS6:
                raise ValueError("monitor component must be one of %s: %r" % (", ".join(COMPONENTS6), comp))
            if not all(0 <= int(v) < n for v, n in zip(ijk, self.shape)):
                raise ValueError("monitor point %r outside the grid %r" % (tuple(ijk), self.shape))
        self.nmon = len(mons)
        self._ijk = torch.tensor([list(map(int, p)) for _, p in mons] or [[0, 0, 0]], dtype=torch.int32, device=dev)
        self._comp = torch.tensor([COMPONENTS6.index(c) for c, _ in mons] or [0], dtype=torch.int32, device=dev)
        self.tstep = 1

    def set_ce(self, ce):
        for q in range(3):
            self.ce[q].copy_(torch.as_tensor(ce[q]).to(device=self.device, dtype=torch.float64))

    def reset(self):
        self.f.zero_()
        for t in self.psi_e + self.psi_h:
            if t is not None:
                t.zero_()
        self.tstep = 1

    @property
    def fields(self):
        return dict(zip(COMPONENTS6, self.f))

    def _args(self):
        nx, ny, nz = self.shape
        g = N.Grid(nx, ny, nz, ny * nz, nz)
        ptr = lambda t: t.data_ptr() if t is not None else None
        f = (C.c_void_p * 6)(*[self.f[q].data_ptr() for q in range(6)])
        ce = (C.c_void_p * 3)(*[self.ce[q].data_ptr() for q in range(3)])
        pe = (C.c_void_p * 6)(*map(ptr, self.psi_e))
        ph = (C.c_void_p * 6)(*map(ptr, self.psi_h))
        return g, f, ce, self.cpml.struct(), pe, ph, self.sources.struct()

    def step(self, n=1, monitor_out=None):
        """Advance n steps; monitor_out (n, nmon) float64 receives the monitor
        values after every step."""
        g, f, ce, cp, pe, ph, src = self._args()
        pts = N.Points(self.nmon, self._ijk.data_ptr(), self._comp.data_ptr())
        L = N.lib()
        with torch.cuda.device(self.device):
            stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            for m in range(n):
                st = L.fdtd_step_unfused_f64(C.byref(g), f, ce, C.byref(cp) if self.cpml.active else None, pe, ph,
                                             C.byref(src), int(self.tstep), stream)
                if st:
                    N.check(st, "fdtd_step_unfused_f64")
                if monitor_out is not None and self.nmon:
                    N.call("fdtd_gather_points_f64", C.byref(g), C.byref(pts), f,
                           C.c_void_p(monitor_out[m].data_ptr()), stream)
                self.tstep += 1

    def run(self, nsteps):
        """Monitor values (nsteps, nmon) of a run from a zero state."""
        self.reset()
        out = torch.zeros((nsteps, max(self.nmon, 1)), dtype=torch.float64, device=self.device)
        self.step(nsteps, out)
        return out[:, :self.nmon]


class SympRun64:
    """FP64 twin of a SymplecticSolver (fdtd_symplectic_stage_f64): the same
    stages, CPML and sources in double precision on the GPU, with the FP32
    solver's coefficients, CPML tables and source amplitudes widened, so the
    two runs discretise the same problem.  Build it from the solver whose
    accuracy it measures; its fields start at zero."""

    def __init__(self, solver):
        self.src32 = solver
        self.shape = solver.shape
        self.device = solver.device
        dev = self.device
        self.f = torch.zeros((6,) + self.shape, dtype=torch.float64, device=dev)
        self.ce = torch.stack([c.double() for c in solver.ce])
        if isinstance(solver.ch, float):
            self.ch_arrays = None
            self.ch = float(np.float32(solver.ch))
        else:
            self.ch_arrays = torch.stack([c.double() for c in solver.ch])
            self.ch = 0.0
        cp = solver.cpml
        self.psi_e = [torch.zeros_like(t, dtype=torch.float64) if t is not None else None for t in cp.psi_e]
        self.psi_h = [torch.zeros_like(t, dtype=torch.float64) if t is not None else None for t in cp.psi_h]
        self.tstep = solver.tstep

    @property
    def fields(self):
        return dict(zip(COMPONENTS6, self.f))

    def step(self, n=1):
        from .symplectic import CL, DL
        s = self.src32
        if s.src_spec and self.tstep + n > s._src_steps:
            s._build_sources(self.tstep + n)
        nx, ny, nz = self.shape
        g = N.Grid(nx, ny, nz, ny * nz, nz)
        ptr = lambda t: t.data_ptr() if t is not None else None
        f = (C.c_void_p * 6)(*[self.f[q].data_ptr() for q in range(6)])
        ce = (C.c_void_p * 3)(*[self.ce[q].data_ptr() for q in range(3)])
        ch = (C.c_void_p * 3)(*[self.ch_arrays[q].data_ptr() for q in range(3)]) if self.ch_arrays is not None else None
        pe = (C.c_void_p * 6)(*map(ptr, self.psi_e))
        ph = (C.c_void_p * 6)(*map(ptr, self.psi_h))
        active = s.cpml.active
        src = s._src.struct()
        L = N.lib()
        w32 = lambda v: float(np.float32(v))   # the FP32 path's coefficient, widened

        def stage(e_or_h, coef, cf, psi, chv):
            cp = C.byref(s.cpml._structs[coef]) if active else None
            st = L.fdtd_symplectic_stage_f64(C.byref(g), cp, int(e_or_h), w32(coef), chv, f, cf,
                                             psi if active else None, stream)
            if st:
                N.check(st, "fdtd_symplectic_stage_f64")

        with torch.cuda.device(self.device):
            stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            for _ in range(n):
                tn = self.tstep
                for sn in range(4):
                    stage(0, CL[sn], ch, ph, self.ch)
                    stage(1, DL[sn], ce, pe, 0.0)
                    if s.src_spec:
                        N.call("fdtd_add_sources_f64", C.byref(g), C.byref(src), 4 * tn + sn,
                               *[C.c_void_p(self.f[q].data_ptr()) for q in range(3)], stream)
                stage(0, CL[4], ch, ph, self.ch)
                self.tstep += 1


def family_errors(f32, f64):
    """Distance of an FP32 run to its FP64 twin, per component: max |a - b| and
    the root-mean-square |a - b|, each divided by the largest |b| (resp. the
    root-mean-square |b|) of the component's field family (E or H).
    Per-component normalisation is meaningless for a component that is zero
    in exact arithmetic (its FP64 value is roundoff)."""
    out = {}
    for fam in (COMPONENTS6[:3], COMPONENTS6[3:]):
        vmax = max(float(f64[k].abs().max()) for k in fam)
        vrms = (sum(float((f64[k] ** 2).sum()) for k in fam) / sum(f64[k].numel() for k in fam)) ** 0.5
        for k in fam:
            d = f32[k].double() - f64[k]
            out[k] = {"max": float(d.abs().max()) / vmax, "rms": float((d ** 2).mean()) ** 0.5 / vrms}
    return out

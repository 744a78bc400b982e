"""Gradient of an FDTD run with respect to the E coefficients (CE = dt/eps).

The reference has no gradient path; this is the reverse-time form of its
2nd-order Yee step with CPML (the step of solver.py).  ``YeeAdjoint`` runs
the forward simulation with the fused kernel, recording

  * the field values at monitor points after every step, and
  * a checkpoint of the whole state (E, H, psi_e, psi_h) every K steps,

and its backward pass walks the segments last to first: it recomputes the K
states of a segment from its checkpoint into K+1 state slots (one fused launch
per step, each writing its own slot), then applies the hand-written adjoint
step (fdtd_adjoint_step_f32) from the last state of the segment down to the
first, accumulating dL/dCE.  With overlap (the default), a second set of
slots lets the recompute of the segment before run on a second stream while
the reverse steps of the current one run.  Memory: ceil(N/K) checkpoints +
(K+1) slots (twice that with overlap).

``fdtd_run(ce, engine)`` is the differentiable call:

    mon, fields = fdtd_run(ce, engine)      # ce: (3, nx, ny, nz), requires_grad
    loss = (mon.double() ** 2).sum()
    loss.backward()                         # ce.grad = dL/dCE (cex, cey, cez)

The gradient with respect to a permittivity map follows through torch from
CE = dt / eps (kuFDTD/v0.2.0/dim3/cpu/matter.py:81-83).
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N
from .cpml import CpmlLayer
from .solver import padded_nz
from .sources import PointSources

__all__ = ["YeeAdjoint", "fdtd_run", "COMPONENTS6"]

COMPONENTS6 = ("ex", "ey", "ez", "hx", "hy", "hz")


class YeeAdjoint:
    """Forward/backward engine for one grid.

    monitors: list of (component, (i, j, k)); component in ex..hz.
    segment: checkpoint interval K (steps).
    grad_region: three slices (a design region): dL/dCE is accumulated only
    there (fdtd_adjoint_step_region_f32) and returned as zero elsewhere; the
    reverse steps then skip the forward-H reads and the accumulator traffic of
    every other cell.  None: every cell.
    overlap: in the backward pass, recompute segment c-1 into a second set of
    state slots on a second stream while the reverse steps of segment c run
    (the same kernels and results; K+1 more slots of device memory).
    """

    def __init__(self, shape, nsteps, npml=0, faces=0x3F, cpml_params=None, sources=(), monitors=(),
                 segment=100, device="cuda", tile=None, grad_region=None, overlap=True):
        nx, ny, nz = (int(v) for v in shape)
        self.shape = (nx, ny, nz)
        self.nsteps = int(nsteps)
        if self.nsteps < 1:
            raise ValueError("nsteps must be positive")
        self.K = max(1, min(int(segment), self.nsteps))
        self.device = torch.device(device)
        dev = self.device
        self.nzp = padded_nz(nz)
        self.cpml = CpmlLayer(self.shape, npml, faces, device=dev, **(cpml_params or {}))
        self.sources = PointSources(self.shape, sources, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.tile = tile
        K = self.K
        # state slots: slot m holds the state after m steps of the current segment
        self.slots = torch.zeros((K + 1, 6, nx, ny, self.nzp), dtype=torch.float32, device=dev)
        self.slot_psi_e = [self._psi_like(self.cpml.psi_e[0]) for _ in range(K + 1)]
        self.psi_h = self.cpml.psi_h
        self._ce = torch.zeros((3, nx, ny, self.nzp), dtype=torch.float32, device=dev)
        mons = list(monitors)
        for comp, ijk in mons:
            if comp not in COMPONENTS6:
                raise ValueError("monitor component must be one of %s: %r" % (", ".join(COMPONENTS6), comp))
            if len(ijk) != 3 or not all(0 <= int(v) < n for v, n in zip(ijk, self.shape)):
                raise ValueError("monitor point %r outside the grid %r" % (tuple(ijk), self.shape))
        self.nmon = len(mons)
        self._mon_ijk = torch.tensor([list(map(int, p)) for _, p in mons] or [[0, 0, 0]],
                                     dtype=torch.int32, device=dev)
        self._mon_comp = torch.tensor([COMPONENTS6.index(c) for c, _ in mons] or [0],
                                      dtype=torch.int32, device=dev)
        self.overlap = bool(overlap)
        # slot sets: set 0 is (slots, slot_psi_e); set 1 (overlapped backward)
        # is allocated by the first backward pass that uses it
        self._sets = [(self.slots, self.slot_psi_e)]
        self._plans = None        # per set: one fused plan per slot pair
        self._ptrs = {}
        self._slots_hold = None   # (run id, segment) whose states slot set 0 holds
        self._run_id = 0
        self._gbox = None
        if grad_region is not None:
            box = []
            for sl, n in zip(grad_region, self.shape):
                a, b, st = sl.indices(n)
                if st != 1 or b <= a:
                    raise ValueError("grad_region needs three non-empty unit-step slices: %r" % (grad_region,))
                box.append((a, b - a))
            self._gbox = (C.c_int64 * 6)(*[v[0] for v in box], *[v[1] for v in box])

    # ------------------------------------------------------------ helpers
    @staticmethod
    def _psi_like(lst):
        return [torch.zeros_like(t) if t is not None else None for t in lst]

    def grid(self):
        nx, ny, nz = self.shape
        return N.Grid(nx, ny, nz, ny * self.nzp, self.nzp)

    def points(self):
        p = N.Points()
        p.n = self.nmon
        p.ijk = self._mon_ijk.data_ptr()
        p.comp = self._mon_comp.data_ptr()
        return p

    def _plan_state(self, m, k=0):
        slots, slot_psi_e = self._sets[k]
        s = N.YeeState()
        for b, slot in ((0, m), (1, m + 1)):
            for q in range(6):
                s.f[b][q] = slots[slot, q].data_ptr()
                e = slot_psi_e[slot][q]
                s.psi_e[b][q] = e.data_ptr() if e is not None else None
        for q in range(6):
            h = self.psi_h[q]
            s.psi_h[q] = h.data_ptr() if h is not None else None
        for q in range(3):
            s.ce[q] = self._ce[q].data_ptr()
        return s

    def plans(self, k=0):
        """One fused plan per slot pair (m -> m+1) of slot set k."""
        if self._plans is None:
            self._plans = {}
        if k not in self._plans:
            g = self.grid()
            cp = self.cpml.struct()
            src = self.sources.struct()
            tile = N.Tile(*(tuple(self.tile or ()) + (0, 0, 0, 0, 0))[:5])
            plans = []
            with torch.cuda.device(self.device):
                for m in range(self.K):
                    h = C.c_void_p()
                    st = self._plan_state(m, k)
                    N.call("fdtd_yee_plan_create", C.byref(h), C.byref(g), C.byref(st), C.byref(cp),
                           C.byref(src), C.byref(tile), C.c_void_p(self.status.data_ptr()), 0, self._stream())
                    plans.append(h)
            self._plans[k] = plans
        return self._plans[k]

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _step_slot(self, m, t, k=0):
        """Fused step from slot m to slot m+1 of set k with step number t."""
        L = N.lib()
        plan = self.plans(k)[m]
        L.fdtd_yee_plan_set_current(plan, 0)
        N.call("fdtd_yee_plan_run", plan, int(t), 1, self._stream())

    def _slot_ptrs(self, k=0):
        """Per-slot pointer arrays (fields, H, E-psi) of slot set k, built once."""
        if k not in self._ptrs:
            slots, slot_psi_e = self._sets[k]
            f, h, pe = [], [], []
            for m in range(self.K + 1):
                f.append((C.c_void_p * 6)(*[slots[m, q].data_ptr() for q in range(6)]))
                h.append((C.c_void_p * 3)(*[slots[m, 3 + q].data_ptr() for q in range(3)]))
                pe.append((C.c_void_p * 6)(*[t.data_ptr() if t is not None else None for t in slot_psi_e[m]]))
            self._ptrs[k] = (f, h, pe, self.grid(), self.points())
        return self._ptrs[k]

    def _gather(self, slot, out_row):
        if not self.nmon:
            return
        f, _, _, g, pts = self._slot_ptrs()
        N.call("fdtd_gather_points_f32", C.byref(g), C.byref(pts), f[slot], C.c_void_p(out_row.data_ptr()),
               self._stream())

    def _segments(self):
        K, N_ = self.K, self.nsteps
        return [(c * K, min(K, N_ - c * K)) for c in range((N_ + K - 1) // K)]

    def set_ce(self, ce):
        nz = self.shape[2]
        self._ce[:, :, :, :nz].copy_(ce.detach().to(device=self.device, dtype=torch.float32))

    def _load(self, ck, k=0):
        state, pe, ph = ck
        slots, slot_psi_e = self._sets[k]
        slots[0].copy_(state)
        for dst, src in zip(slot_psi_e[0], pe):
            if dst is not None:
                dst.copy_(src)
        for dst, src in zip(self.psi_h, ph):
            if dst is not None:
                dst.copy_(src)

    def _checkpoint(self):
        return (self.slots[0].clone(), [t.clone() if t is not None else None for t in self.slot_psi_e[0]],
                [t.clone() if t is not None else None for t in self.psi_h])

    # ------------------------------------------------------------ forward
    def forward(self, ce):
        """Run nsteps from a zero state.  Returns (monitors (nsteps, nmon),
        final fields (6, nx, ny, nz), checkpoints, run id)."""
        nz = self.shape[2]
        self.set_ce(ce)
        self.plans()
        self.slots[0].zero_()
        for t in self.slot_psi_e[0] + self.psi_h:
            if t is not None:
                t.zero_()
        mon = torch.zeros((self.nsteps, max(self.nmon, 1)), dtype=torch.float32, device=self.device)
        checkpoints = []
        segs = self._segments()
        with torch.cuda.device(self.device):
            for c, (t0, L) in enumerate(segs):
                if c > 0:
                    # slot 0 <- last state of the previous segment
                    self.slots[0].copy_(self.slots[segs[c - 1][1]])
                    for dst, src in zip(self.slot_psi_e[0], self.slot_psi_e[segs[c - 1][1]]):
                        if dst is not None:
                            dst.copy_(src)
                checkpoints.append(self._checkpoint())
                for m in range(L):
                    self._step_slot(m, t0 + m + 1)
                    self._gather(m + 1, mon[t0 + m])
        self._run_id += 1
        self._slots_hold = (self._run_id, len(segs) - 1)
        final = self.slots[segs[-1][1], :, :, :, :nz].clone()
        return mon[:, :self.nmon], final, checkpoints, self._run_id

    # ------------------------------------------------------------ backward
    def backward(self, ce, checkpoints, run_id, grad_mon=None, grad_fields=None):
        """dL/dCE (3, nx, ny, nz) for the run that made ``checkpoints``."""
        nx, ny, nz = self.shape
        dev = self.device
        self.set_ce(ce)
        lf = torch.zeros((6, nx, ny, self.nzp), dtype=torch.float32, device=dev)
        if grad_fields is not None:
            lf[:, :, :, :nz].copy_(grad_fields)
        gce = torch.zeros((3, nx, ny, self.nzp), dtype=torch.float32, device=dev)
        lpe = self._psi_like(self.cpml.psi_e[0])
        lph = self._psi_like(self.psi_h)
        we = self._psi_like(self.cpml.psi_e[0])
        wh = self._psi_like(self.psi_h)
        st = N.AdjointState()
        for q in range(6):
            st.lf[q] = lf[q].data_ptr()
            for arr, lst in ((st.lpsi_e, lpe), (st.lpsi_h, lph), (st.w_e, we), (st.w_h, wh)):
                arr[q] = lst[q].data_ptr() if lst[q] is not None else None
        for q in range(3):
            st.grad_ce[q] = gce[q].data_ptr()
        cp = self.cpml.struct()
        ce_p = (C.c_void_p * 3)(*[self._ce[q].data_ptr() for q in range(3)])
        gm = None
        if grad_mon is not None and self.nmon:
            gm = grad_mon.detach().to(device=dev, dtype=torch.float32).contiguous()
        segs = self._segments()
        nseg = len(segs)
        overlap = self.overlap and nseg > 1
        if overlap and len(self._sets) == 1:
            try:
                self._sets.append((torch.zeros_like(self.slots), [self._psi_like(p) for p in self.slot_psi_e]))
            except torch.cuda.OutOfMemoryError:
                overlap = False   # no room for a second slot set: recompute in line
        fn = N.lib().fdtd_adjoint_step_f32 if self._gbox is None else N.lib().fdtd_adjoint_step_region_f32
        extra = () if self._gbox is None else (self._gbox,)
        row = gm.stride(0) * 4 if gm is not None else 0
        base = gm.data_ptr() if gm is not None else 0
        # slot set of segment c: the last segment in set 0 (where the forward
        # run left it), then alternating
        set_of = (lambda c: (nseg - 1 - c) % 2) if overlap else (lambda c: 0)
        with torch.cuda.device(dev):
            main = torch.cuda.current_stream(dev)
            side = torch.cuda.Stream(dev) if overlap else main
            recomputed = [None] * nseg   # event: segment c's states are in its set
            released = {}                # set -> event: the reverse steps using it are done
            if overlap:
                side.wait_stream(main)   # CE, the checkpoints and the forward run's states

            def recompute(c):
                k = set_of(c)
                t0, L = segs[c]
                if k in released:
                    side.wait_event(released[k])
                with torch.cuda.stream(side):
                    self._load(checkpoints[c], k)
                    for m in range(L):
                        self._step_slot(m, t0 + m + 1, k)
                    ev = torch.cuda.Event()
                    ev.record(side)
                recomputed[c] = ev

            if self._slots_hold != (run_id, nseg - 1):
                recompute(nseg - 1)
            for c in range(nseg - 1, -1, -1):
                if overlap and c > 0:
                    recompute(c - 1)     # on the side stream, beside the reverse steps below
                elif not overlap and c < nseg - 1:
                    recompute(c)
                if recomputed[c] is not None:
                    main.wait_event(recomputed[c])
                t0, L = segs[c]
                k = set_of(c)
                _, hps, pes, g, pts = self._slot_ptrs(k)
                gp, cpp, stp = C.byref(g), C.byref(cp), C.byref(st)
                ptsp = C.byref(pts) if gm is not None else None
                stream = C.c_void_p(main.cuda_stream)
                for n in range(L, 0, -1):
                    T = t0 + n
                    mon_ptr = C.c_void_p(base + (T - 1) * row) if gm is not None else None
                    rc = fn(gp, cpp, stp, hps[n - 1], pes[n], ce_p, ptsp, mon_ptr, *extra, stream)
                    if rc:
                        N.check(rc, "fdtd_adjoint_step_f32")
                if overlap:
                    ev = torch.cuda.Event()
                    ev.record(main)
                    released[k] = ev
            if overlap:
                main.wait_stream(side)
        # slot set 0 holds segment 0 now when it is its set, else an older one
        self._slots_hold = (run_id, 0) if set_of(0) == 0 else None
        return gce[:, :, :, :nz]

    def check_status(self):
        v = int(self.status.item())
        if v:
            self.status.zero_()
            N.check(v, "fdtd_yee_plan_run (device status)")

    def close(self):
        if self._plans is not None:
            L = N.lib()
            for plans in self._plans.values():
                for h in plans:
                    L.fdtd_yee_plan_destroy(h)
            self._plans = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _YeeRun(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ce, engine):
        mon, final, cks, run_id = engine.forward(ce)
        ctx.set_materialize_grads(False)
        ctx.engine = engine
        ctx.cks = cks
        ctx.run_id = run_id
        ctx.save_for_backward(ce)
        return mon, final

    @staticmethod
    def backward(ctx, grad_mon, grad_fields):
        (ce,) = ctx.saved_tensors
        g = ctx.engine.backward(ce, ctx.cks, ctx.run_id, grad_mon=grad_mon, grad_fields=grad_fields)
        return g.to(ce.dtype), None


def fdtd_run(ce, engine):
    """Differentiable run: (monitor series (nsteps, nmon), final fields
    (6, nx, ny, nz)) as functions of ce (3, nx, ny, nz)."""
    if not isinstance(engine, YeeAdjoint):
        raise TypeError("engine must be a YeeAdjoint")
    if tuple(ce.shape) != (3,) + engine.shape:
        raise ValueError("ce must have shape (3, %d, %d, %d)" % engine.shape)
    return _YeeRun.apply(ce, engine)

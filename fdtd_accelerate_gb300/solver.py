"""Whole-simulation driver for the 2nd-order Yee step on one GPU.

YeeSolver owns a z-padded, double-buffered device state (E, H, E-psi) plus
the coefficient arrays, the CPML layer and the point sources, and advances
it with the fused kernel (one HBM pass per step, fdtd_yee_plan_* in the C
ABI) or, for checking, with the unfused reference-shaped kernels
(fdtd_step_unfused_f32).  Both give bit-identical results.

Step order and time index follow the reference's loop
(2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:718-742,
KEMP/v0.7_pml/fdtd3d/main.py:296-326): step number t starts at 1 and the
source amplitude used in step t is table[t].
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N
from .cpml import CpmlLayer
from .sources import PointSources

__all__ = ["YeeSolver", "padded_nz", "FIELD_NAMES"]

FIELD_NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


def padded_nz(nz, align=4):
    """z pitch: a multiple of 4 floats keeps rows 16-byte aligned for TMA."""
    return (nz + align - 1) // align * align


class YeeSolver:
    def __init__(self, shape, ce=None, npml=0, faces=0x3F, cpml_params=None, sources=(),
                 device="cuda", tile=None, z_align=4, drude=None, tfsf=None):
        nx, ny, nz = (int(v) for v in shape)
        self.shape = (nx, ny, nz)
        self.device = torch.device(device)
        self.nzp = padded_nz(nz, z_align)
        dev = self.device
        # state[b] : (6, nx, ny, nzp) for buffer b; views give (nx, ny, nz)
        self._state = torch.zeros((2, 6, nx, ny, self.nzp), dtype=torch.float32, device=dev)
        self._ce = torch.zeros((3, nx, ny, self.nzp), dtype=torch.float32, device=dev)
        if ce is None:
            self._ce[:, :, :, :nz] = 0.5
        else:
            for q in range(3):
                self._ce[q, :, :, :nz] = torch.as_tensor(ce[q], dtype=torch.float32, device=dev)
        self.cpml = CpmlLayer(self.shape, npml, faces, device=dev, double_buffer_e=True,
                              **(cpml_params or {}))
        self.sources = PointSources(self.shape, sources, device=dev)
        # optional Drude region (DrudeAde), applied after the E update, before the CPML
        if drude is not None and (tuple(drude.grid_shape) != self.shape or drude.J.device != self._state.device):
            raise ValueError("the Drude region belongs to a %s grid on %s" % (drude.grid_shape, drude.J.device))
        # optional plane-wave source (Tfsf), applied after the E and H CPML
        # corrections (before the point sources) by both steps
        if tfsf is not None and tuple(tfsf.shape) != self.shape:
            raise ValueError("the TFSF source belongs to a %s grid" % (tfsf.shape,))
        self.tfsf = tfsf
        self.drude = drude
        self._drude_struct = drude.struct(both_buffers=True) if drude is not None else None
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._cur = 0
        self.tstep = 1
        self.tile = tile
        self._plan = None

    @property
    def cur(self):
        """Index of the state buffer holding the current fields (and E-psi, J)."""
        return self._cur

    @cur.setter
    def cur(self, value):
        self._cur = int(value)
        if self.drude is not None:
            self.drude.cur = self._cur

    # ------------------------------------------------------------------ views
    def _views(self, b):
        nz = self.shape[2]
        return [self._state[b, q, :, :, :nz] for q in range(6)]

    @property
    def fields(self):
        return dict(zip(FIELD_NAMES, self._views(self.cur)))

    @property
    def ce(self):
        nz = self.shape[2]
        return [self._ce[q, :, :, :nz] for q in range(3)]

    def set_fields(self, **arrays):
        f = self.fields
        for k, v in arrays.items():
            f[k].copy_(torch.as_tensor(v, dtype=torch.float32, device=self.device))

    def load_host(self, fields, ce=None):
        """Copy host arrays (ideally pinned) into the current state and,
        optionally, the E coefficients; stream-ordered on the current stream."""
        f = self.fields
        for k, v in fields.items():
            f[k].copy_(torch.as_tensor(v), non_blocking=True)
        if ce is not None:
            for q in range(3):
                self.ce[q].copy_(torch.as_tensor(ce[q]), non_blocking=True)

    def store_host(self, fields):
        """Copy the current state into host arrays (dict of CPU tensors)."""
        f = self.fields
        for k, v in fields.items():
            v.copy_(f[k], non_blocking=True)

    def grid(self):
        nx, ny, nz = self.shape
        return N.Grid(nx, ny, nz, ny * self.nzp, self.nzp)

    # ------------------------------------------------------------------ fused
    def _state_struct(self):
        s = N.YeeState()
        for b in range(2):
            for q in range(6):
                s.f[b][q] = self._state[b, q].data_ptr()
                e = self.cpml.psi_e[b][q]
                s.psi_e[b][q] = e.data_ptr() if e is not None else None
        for q in range(6):
            h = self.cpml.psi_h[q]
            s.psi_h[q] = h.data_ptr() if h is not None else None
        for q in range(3):
            s.ce[q] = self._ce[q].data_ptr()
        s.drude = C.addressof(self._drude_struct) if self._drude_struct is not None else None
        self._tfsf_struct = self.tfsf.struct() if self.tfsf is not None else None
        s.tfsf = C.addressof(self._tfsf_struct) if self._tfsf_struct is not None else None
        return s

    def plan(self):
        if self._plan is None:
            g = self.grid()
            st = self._state_struct()
            cp = self.cpml.struct()
            src = self.sources.struct()
            tile = N.Tile(*(tuple(self.tile or ()) + (0, 0, 0, 0, 0))[:5])
            h = C.c_void_p()
            with torch.cuda.device(self.device):
                stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
                N.call("fdtd_yee_plan_create", C.byref(h), C.byref(g), C.byref(st), C.byref(cp),
                       C.byref(src), C.byref(tile), C.c_void_p(self.status.data_ptr()), self.cur, stream)
            self._plan = h
        return self._plan

    def plan_info(self):
        """Launch shape chosen for the fused kernel."""
        info = (C.c_int32 * 8)()
        N.call("fdtd_yee_plan_info", self.plan(), info, 8)
        return dict(zip(("tile_y", "stages", "x_chunk", "ctas", "threads", "smem_bytes", "z_band",
                         "launches_per_step"), list(info)))

    def step(self, n=1):
        """Advance n steps with the fused kernel (one launch per step)."""
        if self.tfsf is not None:
            # the plan holds the source table's address: a longer table needs a new plan
            old = self.tfsf.amp.data_ptr()
            self.tfsf.ensure_steps(self.tstep + n)
            if self.tfsf.amp.data_ptr() != old:
                self.close()
        plan = self.plan()
        L = N.lib()
        L.fdtd_yee_plan_set_current(plan, self.cur)
        with torch.cuda.device(self.device):
            stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            N.call("fdtd_yee_plan_run", plan, int(self.tstep), int(n), stream)
        self.cur = L.fdtd_yee_plan_current(plan)
        self.tstep += n

    def step_unfused(self, n=1):
        """Advance n steps in place with the reference-shaped kernels."""
        g = self.grid()
        cp = self.cpml.struct()
        psi = self.cpml.psi_struct(self.cur)
        src = self.sources.struct()
        f = (C.c_void_p * 6)(*[self._state[self.cur, q].data_ptr() for q in range(6)])
        ce = (C.c_void_p * 3)(*[self._ce[q].data_ptr() for q in range(3)])
        with torch.cuda.device(self.device):
            stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            for _ in range(n):
                if self._drude_struct is None and self.tfsf is None:
                    N.call("fdtd_step_unfused_f32", C.byref(g), f, ce, None,
                           C.byref(cp) if self.cpml.active else None, C.byref(psi),
                           C.byref(src), int(self.tstep), stream)
                else:
                    # the reference-shaped calls in the order of
                    # kuFDTD/v0.2.0/dim3/cpu/test/030-drude-cpml.py:88-95
                    E, H = list(f)[:3], list(f)[3:]
                    N.call("fdtd_update_e_f32", C.byref(g), *E, *H, *ce, stream)
                    if self.drude is not None:
                        d = self.drude.struct()
                        N.call("fdtd_drude_update_e_f32", C.byref(g), C.byref(d), *E, *ce, stream)
                    if self.cpml.active:
                        N.call("fdtd_cpml_e_f32", C.byref(g), C.byref(cp), *E, *H, *ce, C.byref(psi), stream)
                    if self.tfsf is not None:
                        self.tfsf.ensure_steps(self.tstep)
                        t = self.tfsf.struct()
                        N.call("fdtd_tfsf_update_e_f32", C.byref(g), C.byref(t), int(self.tstep), *E, stream)
                    N.call("fdtd_add_sources_f32", C.byref(g), C.byref(src), int(self.tstep), *E, stream)
                    N.call("fdtd_update_h_f32", C.byref(g), *E, *H, None, None, None, stream)
                    if self.cpml.active:
                        N.call("fdtd_cpml_h_f32", C.byref(g), C.byref(cp), *E, *H, None, None, None,
                               C.byref(psi), stream)
                    if self.tfsf is not None:
                        N.call("fdtd_tfsf_update_h_f32", C.byref(g), C.byref(t), *H, stream)
                self.tstep += 1

    def test_timeout(self, wait_ns=0, withhold_plane=-1):
        """Set the plan's bounded-wait test hook (fdtd_yee_plan_test_timeout):
        wait_ns > 0 shortens every wait of the fused kernel, withhold_plane >= 0
        makes CTA 0 skip that plane's copies so its wait runs out.  The defaults
        restore normal operation."""
        N.call("fdtd_yee_plan_test_timeout", self.plan(), int(wait_ns), int(withhold_plane))

    def check_status(self):
        """Raise if a bounded device wait expired in an earlier step."""
        v = int(self.status.item())
        if v:
            self.status.zero_()
            N.check(v, "fdtd_yee_plan_run (device status)")

    def psi_e(self):
        return self.cpml.psi_e[self.cur]

    def close(self):
        if self._plan is not None:
            N.lib().fdtd_yee_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""Drude dispersive region: auxiliary differential equation on a sub-box.

Mirrors kuFDTD's DrudeAde (kuFDTD/v0.2.0/dim3/cpu/matter.py:222-314): a box
of (ni, nj, nk) cells at (i0, j0, k0) of the E arrays holds a polarisation
current J and its coefficients per component,

    CJA = (2 - gamma dt) / (2 + gamma dt),  CJB = 4 (dt wp)^2 / (2 + gamma dt)

(evaluated in float32 as matter.py:268-278 does on its 'f' arrays), and after
the E update, before the CPML correction, every box cell takes

    e' = e - ce J;  e = e';  J = CJA J + CJB e'

(kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c:48-93).  `update_e` is the
reference-shaped per-call form (DrudeAde.updateE); passing the region to
YeeSolver applies it inside the fused step.
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N

__all__ = ["DrudeAde", "drude_coefficients"]


def drude_coefficients(pfreq, gamma, dt=0.5):
    """(CJA, CJB) as float32 arrays of the broadcast shape of pfreq, gamma."""
    g = np.asarray(gamma, np.float32)
    w = np.asarray(pfreq, np.float32)
    g, w = np.broadcast_arrays(g, w)
    dt32 = np.float32(dt)
    tmp = np.float32(2) + g * dt32
    cja = (np.float32(2) - g * dt32) / tmp
    cjb = np.float32(4) * (dt32 * w) ** 2 / tmp
    return cja.astype(np.float32), cjb.astype(np.float32)


class DrudeAde:
    """origin (i0, j0, k0) and size (ni, nj, nk) of the box inside a grid of
    `grid_shape`.  Coefficients start as CJA = 1, CJB = 0 (no dispersion)."""

    def __init__(self, grid_shape, origin, size, device="cuda"):
        nx, ny, nz = (int(v) for v in grid_shape)
        i0, j0, k0 = (int(v) for v in origin)
        ni, nj, nk = (int(v) for v in size)
        if min(ni, nj, nk) < 1 or min(i0, j0, k0) < 0 or i0 + ni > nx or j0 + nj > ny or k0 + nk > nz:
            raise ValueError("Drude box %s at %s does not fit the grid %s" % ((ni, nj, nk), (i0, j0, k0),
                                                                               (nx, ny, nz)))
        self.grid_shape = (nx, ny, nz)
        self.origin = (i0, j0, k0)
        self.size = (ni, nj, nk)
        self.device = torch.device(device)
        # two J buffers: the fused step reads buffer cur and writes the other
        # (YeeSolver keeps cur equal to its own state buffer); per-call
        # updates work in place on buffer cur
        self._J = torch.zeros((2, 3, ni, nj, nk), dtype=torch.float32, device=self.device)
        self.cur = 0
        self.cja = torch.ones((3, ni, nj, nk), dtype=torch.float32, device=self.device)
        self.cjb = torch.zeros((3, ni, nj, nk), dtype=torch.float32, device=self.device)

    def set_coeff(self, pfreq, gamma, dt=0.5):
        """pfreq, gamma: scalars, (ni, nj, nk) arrays, or 3-sequences of those
        (one per component x, y, z), in the normalised units of the step (dt)."""
        def per_comp(v):
            if isinstance(v, (list, tuple)) and len(v) == 3:
                return list(v)
            return [v, v, v]
        for q, (w, g) in enumerate(zip(per_comp(pfreq), per_comp(gamma))):
            a, b = drude_coefficients(w, g, dt)
            self.cja[q].copy_(torch.from_numpy(np.array(np.broadcast_to(a, self.size), np.float32)))
            self.cjb[q].copy_(torch.from_numpy(np.array(np.broadcast_to(b, self.size), np.float32)))

    @property
    def J(self):
        """(3, ni, nj, nk) polarisation current of the current buffer."""
        return self._J[self.cur]

    def reset(self):
        self._J.zero_()

    def struct(self, both_buffers=False):
        """fdtd_drude of the current J buffer (per-call form), or with
        both_buffers the two J buffers as j (buffer 0) and j2 (buffer 1) for a
        fused-step plan."""
        d = N.Drude(*self.origin, *self.size)
        for q in range(3):
            d.j[q] = self._J[0 if both_buffers else self.cur][q].data_ptr()
            d.j2[q] = self._J[1][q].data_ptr() if both_buffers else None
            d.cja[q] = self.cja[q].data_ptr()
            d.cjb[q] = self.cjb[q].data_ptr()
        return d

    def update_e(self, ex, ey, ez, cex, cey, cez):
        """One ADE pass on the box (kuFDTD DrudeAde.updateE), in place."""
        from .api import check_field_tensors, grid_of, stream_of
        ts = (ex, ey, ez, cex, cey, cez)
        ref = check_field_tensors(("ex", "ey", "ez", "cex", "cey", "cez"), ts)
        if tuple(ref.shape) != self.grid_shape:
            raise ValueError("Drude box built for a %s grid, fields are %s" % (self.grid_shape, tuple(ref.shape)))
        if ref.device != self.J.device:
            raise ValueError("fields on %s, Drude arrays on %s" % (ref.device, self.J.device))
        g = grid_of(ref)
        d = self.struct()
        with torch.cuda.device(ref.device):
            N.call("fdtd_drude_update_e_f32", C.byref(g), C.byref(d), *[C.c_void_p(t.data_ptr()) for t in ts],
                   stream_of(ref))

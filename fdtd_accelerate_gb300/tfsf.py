"""Total-field/scattered-field plane wave at normal incidence.

Mirrors kuFDTD's Tfsf (kuFDTD/v0.2.0/dim3/tfsf.py:93-244): a 1-D auxiliary
FDTD grid along the propagation axis (Fdtd1d, tfsf.py:14-42: hard source
E[3] = sin(w dt t), two-step-delay ends) carries the incident wave, and
every enabled face of the total-field box corrects the tangential E (after
the E update and its CPML) and H (after the H update and its CPML) by half
the incident field, with the face slices and coefficients of
tfsf.py:140-231.  Oblique incidence is not implemented in the reference
(tfsf.py:120-122, 216-217) and is not offered here either.

Units are the step's normalised ones (dx = 1, c = 1): a wavelength of L
cells gives w dt = 2 pi dt / L (tfsf.py:124, wfreq = 2 pi c / wavelength).
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _native as N

__all__ = ["Tfsf"]

AXES = {"x": 0, "y": 1, "z": 2}


def _faces(apply_direction):
    faces = 0
    for a, d in enumerate(apply_direction):
        d = d or ""
        if "f" in d:
            faces |= 1 << (2 * a)
        if "b" in d:
            faces |= 1 << (2 * a + 1)
    return faces


class Tfsf:
    """shape: grid (nx, ny, nz); pt1, pt2: corners of the total-field box as
    kuFDTD's Tfsf takes them (None: 1 and n-2); apply_direction: per axis 'f',
    'b', 'fb' or ''; propagation_direction: ('normal', 'x'|'y'|'z');
    polarization_angle in radians; wavelength in cells; steps: length of the
    source table (grown on demand)."""

    def __init__(self, shape, pt1, pt2, apply_direction=("fb", "fb", "fb"), wavelength=20.0,
                 propagation_direction=("normal", "x"), polarization_angle=0.0, dt=0.5, steps=1024,
                 device="cuda"):
        if propagation_direction[0] != "normal":
            raise NotImplementedError("oblique incidence: the reference implements normal incidence only")
        if propagation_direction[1] not in AXES:
            raise ValueError("propagation axis must be 'x', 'y' or 'z': %r" % (propagation_direction[1],))
        n = [int(v) for v in shape]
        p1 = [1 if v is None else int(v) for v in pt1]
        p2 = [n[a] - 2 if v is None else int(v) for a, v in enumerate(pt2)]
        p2 = [v + 1 for v in p2]                      # tfsf.py:100
        for a in range(3):
            if p1[a] < 1 or p2[a] > n[a] - 1 or p2[a] < p1[a] + 1:
                raise ValueError("TFSF box %s..%s does not fit the %s grid with a cell to spare" %
                                 (tuple(p1), tuple(v - 1 for v in p2), tuple(n)))
        self.shape = tuple(n)
        self.p1, self.p2 = p1, p2
        self.faces = _faces(apply_direction)
        self.axis = AXES[propagation_direction[1]]
        self.angle = float(polarization_angle)
        self.wdt = 2.0 * math.pi * float(dt) / float(wavelength)
        self.device = torch.device(device)
        n1d = p2[self.axis] - p1[self.axis] + 11
        self.e1d = torch.zeros(n1d, dtype=torch.float32, device=self.device)
        self.h1d = torch.zeros(n1d, dtype=torch.float32, device=self.device)
        self.abc = torch.zeros(4, dtype=torch.float32, device=self.device)
        self._set_table(steps)

    def _set_table(self, steps):
        t = np.arange(int(steps) + 1, dtype=np.float64)
        amp = np.array([math.sin(self.wdt * v) for v in t], np.float32)  # sin(wfreq*dt*tstep), tfsf.py:38
        self.amp = torch.from_numpy(amp).to(self.device)

    def ensure_steps(self, last_step):
        if last_step >= self.amp.numel():
            self._set_table(max(int(last_step) + 1, 2 * self.amp.numel()))

    def reset(self):
        self.e1d.zero_()
        self.h1d.zero_()
        self.abc.zero_()

    def struct(self):
        t = N.Tfsf()
        for a in range(3):
            t.p1[a] = self.p1[a]
            t.p2[a] = self.p2[a]
        t.faces, t.axis, t.angle = self.faces, self.axis, self.angle
        t.e1d, t.h1d, t.abc = self.e1d.data_ptr(), self.h1d.data_ptr(), self.abc.data_ptr()
        t.amp, t.namp = self.amp.data_ptr(), self.amp.numel()
        return t

    def _call(self, fn, fields, *extra):
        from .api import check_field_tensors, grid_of, stream_of
        ref = check_field_tensors(("f0", "f1", "f2"), fields)
        if tuple(ref.shape) != self.shape:
            raise ValueError("TFSF built for a %s grid, fields are %s" % (self.shape, tuple(ref.shape)))
        g = grid_of(ref)
        st = self.struct()
        with torch.cuda.device(ref.device):
            N.call(fn, C.byref(g), C.byref(st), *extra, *[C.c_void_p(f.data_ptr()) for f in fields], stream_of(ref))

    def update_e(self, ex, ey, ez, tstep):
        """Tfsf.updateE(tstep): the 1-D E step, then the E face corrections."""
        self.ensure_steps(tstep)
        self._call("fdtd_tfsf_update_e_f32", (ex, ey, ez), C.c_int64(int(tstep)))

    def update_h(self, hx, hy, hz):
        """Tfsf.updateH(): the 1-D H step, then the H face corrections."""
        self._call("fdtd_tfsf_update_h_f32", (hx, hy, hz))

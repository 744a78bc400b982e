"""CPML coefficient tables and psi storage (host set-up + device state).

Normalised units: dx = 1, c = 1, eps0 = mu0 = eta0 = 1, so the Courant
number S = dt and the E coefficient is ce = dt / eps_r (0.5 / eps_r for
S = 0.5, as in kuFDTD/v0.2.0/dim3/cpu/matter.py:81-83).

Grading (depth rho in cells from the inner PML interface, P slab cells):
    sigma(rho) = sigma_max (rho/P)^m
    kappa(rho) = 1 + (kappa_max - 1) (rho/P)^m
    alpha(rho) = alpha_max (1 - rho/P)^m_alpha
    b = exp(-(sigma/kappa + alpha) dt)
    a = sigma / (sigma kappa + alpha kappa^2) (b - 1)
    km1 = 1/kappa - 1
    sigma_max = -(m + 1) ln(R) / (2 eta0 P dx)
kappa/sigma/b/a follow kuFDTD/before_CUDA/v0.3.0/boundary/cpml.py:126-136,
alpha grading KEMP/v0.7_pml/fdtd3d/naive/pml.py:35-36; sigma_max is taken
from the target reflection R instead of the fixed
kuFDTD/v0.2.0/dim3/cpu/cpml.py:109 expression.

Slab layout: slab index s < P is the front slab (node s+1, depth P-s-1/2
for E nodes, P-s for H nodes); s >= P the back slab (E node n-P-1+(s-P),
depth s-P+1/2; H node n-P+(s-P), depth s-P+1) -- the index ranges of
kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c:59-60,127-128.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _native as N

__all__ = ["cpml_tables", "sigma_max_from_reflection", "parse_faces", "CpmlLayer"]


def sigma_max_from_reflection(npml, m=4, R=1e-8, dx=1.0, eta0=1.0):
    return -(m + 1) * math.log(R) / (2.0 * eta0 * npml * dx)


def cpml_tables(npml, m=4, R=1e-8, kappa_max=5.0, alpha_max=0.05, m_alpha=1, dt=0.5):
    """FP64 tables (2*npml entries each): b_e, a_e, km1_e, b_h, a_h, km1_h."""
    P = int(npml)
    if P <= 0:
        return {k: np.zeros(0) for k in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}
    smax = sigma_max_from_reflection(P, m, R)
    s = np.arange(P, dtype=np.float64)
    depth = {"e": np.concatenate([P - s - 0.5, s + 0.5]), "h": np.concatenate([P - s, s + 1.0])}
    out = {}
    for tag, d in depth.items():
        x = d / P
        sig = smax * x ** m
        kap = 1.0 + (kappa_max - 1.0) * x ** m
        alp = alpha_max * (1.0 - x) ** m_alpha
        b = np.exp(-(sig / kap + alp) * dt)
        den = sig * kap + alp * kap * kap
        a = np.where(den > 0, sig / np.where(den > 0, den, 1.0) * (b - 1.0), 0.0)
        out["b_" + tag] = b
        out["a_" + tag] = a
        out["km1_" + tag] = 1.0 / kap - 1.0
    return out


def parse_faces(directions):
    """Faces bitmask from per-axis strings: 'f'/'-' front, 'b'/'+' back
    (kuFDTD apply_direction ('fb','fb','fb'), KEMP directions ('+-', ...))."""
    if isinstance(directions, int):
        return directions & 0x3F
    if len(directions) != 3:
        raise ValueError("directions must have one entry per axis")
    faces = 0
    for a, d in enumerate(directions):
        if not isinstance(d, str) or set(d) - set("fb+-"):
            raise ValueError("direction %r must use 'f'/'b' or '-'/'+'" % (d,))
        if "f" in d or "-" in d:
            faces |= 1 << (2 * a)
        if "b" in d or "+" in d:
            faces |= 1 << (2 * a + 1)
    return faces


class CpmlLayer:
    """Device CPML state for one grid: FP32 tables and psi slabs.

    npml: int or (Px, Py, Pz); faces: bitmask or per-axis direction strings.
    Axes whose faces are both off get no slabs.
    """

    def __init__(self, shape, npml, faces=0x3F, m=4, R=1e-8, kappa_max=5.0, alpha_max=0.05,
                 m_alpha=1, dt=0.5, device="cuda", double_buffer_e=False):
        nx, ny, nz = (int(v) for v in shape)
        self.shape = (nx, ny, nz)
        if isinstance(npml, int):
            npml = (npml, npml, npml)
        faces = parse_faces(faces)
        npml = [int(p) if (faces >> (2 * a)) & 3 else 0 for a, p in enumerate(npml)]
        for a, (p, n) in enumerate(zip(npml, self.shape)):
            if p < 0 or (p > 0 and n < 2 * p + 2):
                raise ValueError("axis %d: %d CPML cells need at least %d cells, grid has %d"
                                 % (a, p, 2 * p + 2, n))
        self.npml = tuple(npml)
        self.faces = faces
        self.params = dict(m=m, R=R, kappa_max=kappa_max, alpha_max=alpha_max, m_alpha=m_alpha, dt=dt)
        self.device = torch.device(device)
        self.tables64 = [cpml_tables(p, **self.params) for p in self.npml]
        self.tables = [{k: torch.tensor(v, dtype=torch.float32, device=self.device) for k, v in t.items()}
                       for t in self.tables64]
        pshapes = [(2 * npml[0], ny, nz), (nx, 2 * npml[1], nz), (nx, ny, 2 * npml[2])]
        nbuf = 2 if double_buffer_e else 1

        def zeros(a):
            return torch.zeros(pshapes[a], dtype=torch.float32, device=self.device) if npml[a] else None

        self.psi_e = [[zeros(a) for a in range(3) for _ in range(2)] for _ in range(nbuf)]
        self.psi_h = [zeros(a) for a in range(3) for _ in range(2)]
        self._keep = []

    @property
    def active(self):
        return any(self.npml)

    def struct(self):
        c = N.Cpml()
        for a in range(3):
            c.npml[a] = self.npml[a]
        c.faces = self.faces
        for a in range(3):
            t = self.tables[a]
            for key in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h"):
                getattr(c, key)[a] = t[key].data_ptr() if self.npml[a] else None
        return c

    def psi_struct(self, buf=0):
        p = N.Psi()
        for q in range(6):
            p.e[q] = self.psi_e[buf][q].data_ptr() if self.psi_e[buf][q] is not None else None
            p.h[q] = self.psi_h[q].data_ptr() if self.psi_h[q] is not None else None
        return p

    def reset(self):
        for buf in self.psi_e:
            for t in buf:
                if t is not None:
                    t.zero_()
        for t in self.psi_h:
            if t is not None:
                t.zero_()

    # -- reference-shaped per-call updates (kuFDTD CpmlNonKappa.updateE/H,
    #    kuFDTD/v0.2.0/dim3/cpu/cpml.py:129-203; KEMP Pml.update_e/h) -------
    def update_e(self, ex, ey, ez, hx, hy, hz, cex, cey, cez):
        from .api import check_field_tensors, grid_of, stream_of
        ts = (ex, ey, ez, hx, hy, hz, cex, cey, cez)
        ref = check_field_tensors(("ex", "ey", "ez", "hx", "hy", "hz", "cex", "cey", "cez"), ts)
        self._check_shape(ref)
        g = grid_of(ref)
        c = self.struct()
        psi = self.psi_struct(0)
        with torch.cuda.device(ref.device):
            N.call("fdtd_cpml_e_f32", C.byref(g), C.byref(c), *[C.c_void_p(t.data_ptr()) for t in ts],
                   C.byref(psi), stream_of(ref))

    def update_h(self, ex, ey, ez, hx, hy, hz, chx=None, chy=None, chz=None):
        from .api import check_field_tensors, grid_of, stream_of
        ts = [ex, ey, ez, hx, hy, hz]
        names = ["ex", "ey", "ez", "hx", "hy", "hz"]
        if chx is not None:
            ts += [chx, chy, chz]
            names += ["chx", "chy", "chz"]
        ref = check_field_tensors(names, ts)
        self._check_shape(ref)
        g = grid_of(ref)
        c = self.struct()
        psi = self.psi_struct(0)
        ptrs = [C.c_void_p(t.data_ptr()) for t in (ex, ey, ez, hx, hy, hz)]
        ptrs += [C.c_void_p(t.data_ptr()) if t is not None else None for t in (chx, chy, chz)]
        with torch.cuda.device(ref.device):
            N.call("fdtd_cpml_h_f32", C.byref(g), C.byref(c), *ptrs, C.byref(psi), stream_of(ref))

    def _check_shape(self, t):
        if tuple(t.shape) != self.shape:
            raise ValueError("CPML layer built for %s, fields are %s" % (self.shape, tuple(t.shape)))

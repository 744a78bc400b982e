"""Seeded synthetic workloads (the reference publishes no datasets).

Positions of the staggered components in cell units (the Yee grid implied
by the forward E / backward H differences of 2nd_order-Yee/Numpy/fdtd3d.py):
    ex[i,j,k] at (i, j+1/2, k+1/2)   ey at (i+1/2, j, k+1/2)   ez at (i+1/2, j+1/2, k)
Permittivity is sampled at those points (as kuFDTD/v0.2.0/dim3/cpu/matter.py:74-79
does) and CE = dt / eps_r with dt = 0.5 (matter.py:81-83).

Workloads
  plain128   128^3, PEC walls, vacuum, Ez point source at the centre,
             Gaussian-modulated sine (f dt = 0.05, width 30 steps, t0 = 150)
  cpml1024   1024 x 1024 x 512, 12-cell CPML on all faces (m=4, R=1e-8,
             kappa_max=5, alpha_max=0.05), 200 seeded spheres (radius 5..40,
             eps_r U[1,12]), 6 seeded dipoles (delays t0 in [100, 300])
  batched64  64 independent grids, each axis drawn from {32, 48, ..., 192},
             8-cell CPML, 10 spheres per grid (radius 2..n_min/6, eps_r
             U[1,8]), Ez source at the centre, 500 steps
  adjoint256 256 x 256 x 128, 12-cell CPML, a centred 128 x 128 x 64 design
             region of eps_r U[1,12] per cell in vacuum, an Ez line source
             along z at x = npml+3, 16 seeded Ez probes in the far side of the
             region, loss = sum over steps and probes of Ez^2, 3000 steps,
             checkpoints every 100
"""
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from .sources import gaussian_sine

__all__ = ["Workload", "plain128", "cpml1024", "batched64", "adjoint256", "scaled", "paint_spheres", "ce_from_spheres",
           "random_spheres", "random_dipoles", "symp512_solver", "STAGGER"]

# offsets of (ex, ey, ez) sample points from (i, j, k)
STAGGER = ((0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0))


@dataclass
class Workload:
    name: str
    shape: tuple
    steps: int
    npml: int = 0
    spheres: list = field(default_factory=list)   # (cx, cy, cz, r, eps_r)
    dipoles: list = field(default_factory=list)   # (comp, (i, j, k), t0)
    seed: int = 0
    pulse_width: float = 30.0
    pulse_freq: float = 0.05
    dt: float = 0.5

    @property
    def cells(self):
        return int(np.prod(self.shape))

    def source_list(self, nsteps=None):
        """(comp, ijk, FP64 amplitude table indexed by step number 0..nsteps)."""
        n = self.steps if nsteps is None else nsteps
        t = np.arange(n + 1, dtype=np.float64)
        return [(c, ijk, gaussian_sine(t, t0, self.pulse_width, self.pulse_freq)) for c, ijk, t0 in self.dipoles]


def random_spheres(rng, shape, count, rmin, rmax, eps_lo, eps_hi):
    out = []
    for _ in range(count):
        c = [float(rng.uniform(0, n)) for n in shape]
        r = int(rng.integers(rmin, rmax + 1))
        eps = float(rng.uniform(eps_lo, eps_hi))
        out.append((c[0], c[1], c[2], r, eps))
    return out


def random_dipoles(rng, shape, count, margin, t0_lo=100.0, t0_hi=300.0):
    out = []
    for _ in range(count):
        ijk = tuple(int(rng.integers(margin, n - margin)) for n in shape)
        comp = ("ex", "ey", "ez")[int(rng.integers(0, 3))]
        out.append((comp, ijk, float(rng.uniform(t0_lo, t0_hi))))
    return out


def plain128(steps=1000):
    return Workload("plain 2nd-order Yee 128x128x128 PEC vacuum", (128, 128, 128), steps, npml=0,
                    dipoles=[("ez", (64, 64, 64), 150.0)])


def cpml1024(steps=2000, shape=(1024, 1024, 512), seed=20261203, nspheres=200, npml=12, ndipoles=6):
    rng = np.random.default_rng(seed)
    spheres = random_spheres(rng, shape, nspheres, 5, 40, 1.0, 12.0)
    dipoles = random_dipoles(rng, shape, ndipoles, npml + 2)
    return Workload("Yee+CPML %dx%dx%d, %d-cell CPML, %d spheres, %d dipoles" % (*shape, npml, nspheres, ndipoles),
                    tuple(shape), steps, npml=npml, spheres=spheres, dipoles=dipoles, seed=seed)


def batched64(nsims=64, steps=500, seed=20261204, sizes=tuple(range(32, 193, 16)), npml=8, nspheres=10):
    """Ragged batch: per-axis sizes drawn independently, per-grid spheres."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(nsims):
        shape = tuple(int(rng.choice(sizes)) for _ in range(3))
        rmax = max(2, min(shape) // 6)
        spheres = random_spheres(rng, shape, nspheres, 2, rmax, 1.0, 8.0)
        centre = tuple(n // 2 for n in shape)
        out.append(Workload("batched grid %d: %dx%dx%d" % ((s,) + shape), shape, steps, npml=npml,
                            spheres=spheres, dipoles=[("ez", centre, 150.0)], seed=seed))
    return out


@dataclass
class AdjointWorkload:
    name: str
    shape: tuple
    steps: int
    npml: int
    eps: torch.Tensor          # (nx, ny, nz) eps_r per cell (CE = dt/eps for all three components)
    design: tuple               # slices of the design region
    sources: list               # (comp, ijk, FP64 table indexed by step number)
    monitors: list              # (comp, ijk)
    segment: int = 100
    dt: float = 0.5


def adjoint256(steps=3000, shape=(256, 256, 128), region=(128, 128, 64), npml=12, nprobes=16, seed=20261205,
               segment=100):
    """Inverse-design style run: gradient of a probe loss w.r.t. the permittivity of a design region."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    lo = [(n - r) // 2 for n, r in zip(shape, region)]
    design = tuple(slice(l, l + r) for l, r in zip(lo, region))
    eps = torch.ones(shape, dtype=torch.float32)
    eps[design] = torch.from_numpy(rng.uniform(1.0, 12.0, size=region).astype(np.float32))
    t = np.arange(steps + 1, dtype=np.float64)
    amp = gaussian_sine(t, 150.0, 30.0, 0.05)
    x_src = npml + 3
    sources = [("ez", (x_src, ny // 2, k), amp) for k in range(npml + 1, nz - npml - 1)]
    # probes in the far quarter (in x) of the design region
    x0 = lo[0] + 3 * region[0] // 4
    probes = []
    while len(probes) < nprobes:
        p = (int(rng.integers(x0, lo[0] + region[0])), int(rng.integers(lo[1], lo[1] + region[1])),
             int(rng.integers(lo[2], lo[2] + region[2])))
        if p not in probes:
            probes.append(p)
    return AdjointWorkload("adjoint %dx%dx%d, %d-cell CPML, design %dx%dx%d eps U[1,12], Ez line source, "
                           "%d Ez probes, %d steps" % (*shape, npml, *region, nprobes, steps),
                           tuple(shape), steps, npml, eps, design, sources, [("ez", p) for p in probes], segment)


def symp512_solver(shape=(512, 512, 512), device="cuda", max_steps=0, npml=10, seed=20261206, fused=True):
    """The 4th-order workload: 512^3, 10-cell CPML, 60 seeded spheres (radius
    5..40, eps_r U[1,4]), ce = (S/24)/eps_r, ch = S/24, an Ez dipole at the
    centre with the Gaussian-modulated sine (f dt = 0.05, width 30, t0 = 150)
    evaluated at the stage times."""
    from .symplectic import COURANT, SymplecticSolver
    shape = tuple(shape)
    rng = np.random.default_rng(seed)
    spheres = random_spheres(rng, shape, 60, 5, 40, 1.0, 4.0)
    ce = [(c * np.float32(COURANT / 24 / 0.5)) for c in ce_from_spheres(shape, spheres, device=device)]
    src = [("ez", tuple(n // 2 for n in shape),
            lambda t: float(np.sin(2 * np.pi * 0.05 * t) * np.exp(-0.5 * ((t - 150.0) / 30.0) ** 2)))]
    return SymplecticSolver(shape, ce=ce, npml=npml, sources=src, device=device, max_steps=max_steps, fused=fused)


def scaled(work, shape, steps=None):
    """Same construction at another size (spheres scaled with the grid)."""
    f = [a / b for a, b in zip(shape, work.shape)]
    sph = [(cx * f[0], cy * f[1], cz * f[2], max(1, int(round(r * min(f)))), e) for cx, cy, cz, r, e in work.spheres]
    dip = [(c, tuple(min(max(int(v * s), work.npml + 2), n - work.npml - 3) for v, s, n in zip(ijk, f, shape)), t0)
           for c, ijk, t0 in work.dipoles]
    return Workload(work.name + " (scaled to %dx%dx%d)" % tuple(shape), tuple(shape),
                    work.steps if steps is None else steps, npml=work.npml, spheres=sph, dipoles=dip,
                    seed=work.seed, pulse_width=work.pulse_width, pulse_freq=work.pulse_freq, dt=work.dt)


def paint_spheres(shape, spheres, offset, device="cpu", dtype=torch.float32):
    """eps_r sampled at grid points (i, j, k) + offset; spheres painted in order."""
    nx, ny, nz = shape
    eps = torch.ones(shape, dtype=dtype, device=device)
    for cx, cy, cz, r, e in spheres:
        lo = [max(0, int(math.floor(c - o - r))) for c, o in zip((cx, cy, cz), offset)]
        hi = [min(n, int(math.ceil(c - o + r)) + 1) for c, o, n in zip((cx, cy, cz), offset, shape)]
        if any(h <= l for l, h in zip(lo, hi)):
            continue
        x = torch.arange(lo[0], hi[0], device=device, dtype=torch.float64) + offset[0] - cx
        y = torch.arange(lo[1], hi[1], device=device, dtype=torch.float64) + offset[1] - cy
        z = torch.arange(lo[2], hi[2], device=device, dtype=torch.float64) + offset[2] - cz
        d2 = x[:, None, None] ** 2 + y[None, :, None] ** 2 + z[None, None, :] ** 2
        inside = d2 <= float(r) ** 2
        sub = eps[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        sub[inside] = e
    return eps


def ce_from_spheres(shape, spheres, dt=0.5, device="cpu"):
    """(cex, cey, cez) = dt / eps_r at the staggered component points, FP32."""
    out = []
    for off in STAGGER:
        eps = paint_spheres(shape, spheres, off, device=device, dtype=torch.float64)
        out.append((dt / eps).to(torch.float32))
    return out

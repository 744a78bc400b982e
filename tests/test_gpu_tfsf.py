"""Plane-wave TFSF source (normal incidence) on the GPU against the oracle's
restatement of kuFDTD/v0.2.0/dim3/tfsf.py, bit for bit: the 1-D auxiliary
grid, the face corrections of every axis and polarisation, inside a full
step with CPML and a point source."""
import math

import numpy as np
import pytest
import torch

import oracle
from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


@pytest.fixture(scope="module")
def F():
    import fdtd_accelerate_gb300 as F
    F.build()
    return F


def _host(t):
    return t.detach().cpu().numpy()


def _tables(npml):
    t = [oracle.cpml_tables(p) for p in npml]
    return {key: [t[a][key] if npml[a] else None for a in range(3)]
            for key in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}


@pytest.mark.parametrize("shape,npml,pt1,pt2,apply,axis,angle", [
    ((40, 34, 36), 6, (10, 9, 9), (29, 24, 26), ("fb", "fb", "fb"), "x", 0.0),
    ((40, 34, 36), 6, (10, 9, 9), (29, 24, 26), ("fb", "fb", "fb"), "y", 0.6),
    ((40, 34, 36), 6, (10, 9, 9), (29, 24, 26), ("fb", "fb", "fb"), "z", 1.1),
    ((30, 33, 40), 0, (3, None, 5), (25, None, 30), ("f", "", "fb"), "z", 0.3),   # open y, PEC walls
    ((36, 30, 31), 5, (8, 8, 8), (27, 21, 22), ("b", "fb", "f"), "x", 2.0),
])
@pytest.mark.parametrize("fused", [False, True])
def test_step_with_tfsf_bit_exact(F, shape, npml, pt1, pt2, apply, axis, angle, fused):
    """Unfused (reference-shaped calls) and fused step with the plane wave,
    CPML and a point source inside the box, against the oracle."""
    rng = np.random.default_rng(17)
    ce = [(0.5 / rng.uniform(1.0, 3.0, shape)).astype(np.float32) for _ in range(3)]
    init = {k: (0.05 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    nsteps = 14
    t = np.arange(nsteps + 2, dtype=np.float64)
    sources = [("ez", (shape[0] // 3, shape[1] // 2, shape[2] // 2), F.gaussian_sine(t, 3.0, 2.0, 0.1))]
    src = F.Tfsf(shape, pt1, pt2, apply, wavelength=12.0, propagation_direction=("normal", axis),
                 polarization_angle=angle, steps=4)
    faces = [("f" in (apply[a] or "")) if s == 0 else ("b" in (apply[a] or "")) for a in range(3) for s in range(2)]
    ref = oracle.TfsfNormal(shape, pt1, pt2, faces, "xyz".index(axis), angle, src.wdt)
    fields = {k: init[k].copy() for k in NAMES}
    fields.update(cex=ce[0], cey=ce[1], cez=ce[2])
    sim = oracle.OracleSim(fields, (npml,) * 3, 0x3F, _tables((npml,) * 3) if npml else None,
                           [(c, ijk, a.astype(np.float32)) for c, ijk, a in sources], tfsf=ref)
    sim.step(nsteps)
    s = F.YeeSolver(shape, ce=ce, npml=npml, sources=sources, tfsf=src)
    s.set_fields(**init)
    if fused:
        s.step(5)
        s.step(nsteps - 5)          # two plan runs: the 1-D grid carries over
        assert s.plan_info()["launches_per_step"] == (4 if npml else 2)
    else:
        s.step_unfused(nsteps)
    torch.cuda.synchronize()
    s.check_status()
    for k in NAMES:
        np.testing.assert_array_equal(_host(s.fields[k]), sim.f[k], err_msg=k)
    np.testing.assert_array_equal(_host(src.e1d), ref.E)
    np.testing.assert_array_equal(_host(src.h1d), ref.H)
    np.testing.assert_array_equal(_host(src.abc), np.array(ref.abc, np.float32))


def test_tfsf_plane_wave_stays_in_the_box(F):
    """Vacuum, all six faces: the total-field box carries the wave, the
    scattered-field region outside it stays at the FP32 rounding floor."""
    shape = (48, 40, 40)
    p1, p2 = (10, 12, 12), (37, 27, 27)
    src = F.Tfsf(shape, p1, p2, wavelength=16.0, propagation_direction=("normal", "x"), polarization_angle=0.4,
                 steps=80)
    s = F.YeeSolver(shape, tfsf=src)
    s.step_unfused(70)
    torch.cuda.synchronize()
    e = torch.sqrt(sum(s.fields[k].double() ** 2 for k in ("ex", "ey", "ez"))).cpu().numpy()
    inside = e[p1[0] + 1:p2[0], p1[1] + 1:p2[1], p1[2] + 1:p2[2]].max()
    out = np.ones(shape, bool)
    out[p1[0] - 2:p2[0] + 3, p1[1] - 2:p2[1] + 3, p1[2] - 2:p2[2] + 3] = False
    assert inside > 0.5
    assert e[out].max() < 1e-5 * inside


def test_fused_plan_refusals(F):
    """A box whose faces come within P+2 cells of a CPML slab, and a plane wave
    in a batched plan, are refused (the unfused step still takes the first)."""
    shape = (40, 34, 36)
    src = F.Tfsf(shape, (7, 9, 9), (29, 24, 26))        # x front face at 6 < P + 2
    s = F.YeeSolver(shape, npml=6, tfsf=src)
    with pytest.raises(NotImplementedError):           # FDTD_ERR_UNSUPPORTED
        s.step(1)
    s.step_unfused(2)
    src2 = F.Tfsf(shape, (10, 9, 9), (29, 24, 26))
    with pytest.raises(NotImplementedError):
        F.BatchSolver([F.YeeSolver(shape, npml=6, tfsf=src2), F.YeeSolver((20, 20, 20))]).step(1)


def test_tfsf_arguments(F):
    with pytest.raises(ValueError):
        F.Tfsf((20, 20, 20), (0, 5, 5), (10, 10, 10))          # no cell to spare in front
    with pytest.raises(ValueError):
        F.Tfsf((20, 20, 20), (5, 5, 5), (10, 10, 19))          # p2 + 1 past the last cell
    with pytest.raises(NotImplementedError):
        F.Tfsf((20, 20, 20), (5, 5, 5), (10, 10, 10), propagation_direction=("oblique", 0.1, 0.2))


def test_tfsf_matches_reference_golden(F, golden_dir):
    """The per-call GPU TFSF reproduces the reference's own Tfsf outputs
    (tests/golden/tfsf_kufdtd.npz: 12 updateE/updateH pairs from zero fields)."""
    import os
    g = np.load(os.path.join(golden_dir, "tfsf_kufdtd.npz"))
    p1, p2 = [tuple(int(v) for v in r) for r in g["pt"]]
    shape = g["c0_out_ex"].shape
    wavelength = 2 * math.pi * 0.5 / float(g["wdt"])
    for n in range(int(g["ncases"])):
        t = "c%d_" % n
        m = g[t + "meta"]
        apply = tuple(("f" if v & 1 else "") + ("b" if v & 2 else "") for v in m[1:])
        src = F.Tfsf(shape, p1, p2, apply, wavelength=wavelength, propagation_direction=("normal", "xyz"[int(m[0])]),
                     steps=16)
        assert src.wdt == float(g["wdt"])
        f = {k: torch.zeros(shape, dtype=torch.float32, device="cuda") for k in NAMES}
        for step in range(1, 13):
            src.update_e(f["ex"], f["ey"], f["ez"], step)
            src.update_h(f["hx"], f["hy"], f["hz"])
        torch.cuda.synchronize()
        for k in NAMES:
            np.testing.assert_array_equal(_host(f[k]), g[t + "out_" + k], err_msg="case %d %s" % (n, k))
        np.testing.assert_array_equal(_host(src.e1d), g[t + "e1d"])

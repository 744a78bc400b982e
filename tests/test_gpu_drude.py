"""Drude dispersive region (auxiliary differential equation) on the GPU:
the per-call kernel against the reference's own drude_ade.update_e outputs
(tests/golden/drude_kufdtd.npz), and the fused and unfused steps with a Drude
box, CPML and sources against the oracle, bit for bit."""
import os

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


def test_drude_kernel_matches_reference_golden(F, golden_dir):
    g = np.load(os.path.join(golden_dir, "drude_kufdtd.npz"))
    for n in range(int(g["ncases"])):
        t = "c%d_" % n
        m = g[t + "meta"]
        org, box = tuple(int(v) for v in m[:3]), tuple(int(v) for v in m[3:])
        E = [torch.from_numpy(g[t + "in_" + k]).cuda() for k in ("ex", "ey", "ez")]
        CE = [torch.from_numpy(g[t + "in_c" + k]).cuda() for k in ("ex", "ey", "ez")]
        d = F.DrudeAde(E[0].shape, org, box)
        for q, a in enumerate("xyz"):
            d.J[q].copy_(torch.from_numpy(g[t + "in_j" + a]))
            d.cja[q].copy_(torch.from_numpy(g[t + "in_cja" + a]))
            d.cjb[q].copy_(torch.from_numpy(g[t + "in_cjb" + a]))
        for _ in range(3):
            d.update_e(*E, *CE)
        torch.cuda.synchronize()
        for q, k in enumerate(("ex", "ey", "ez")):
            np.testing.assert_array_equal(_host(E[q]), g[t + "out_" + k], err_msg="case %d %s" % (n, k))
            np.testing.assert_array_equal(_host(d.J[q]), g[t + "out_j" + k[1]], err_msg="case %d J%s" % (n, k[1]))


def _tables(npml):
    t = [oracle.cpml_tables(p) for p in npml]
    return {key: [t[a][key] if npml[a] else None for a in range(3)]
            for key in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}


def _case(F, shape, npml, origin, size, seed):
    rng = np.random.default_rng(seed)
    ce = [(0.5 / rng.uniform(1.0, 4.0, shape)).astype(np.float32) for _ in range(3)]
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    wp = [rng.uniform(0.05, 0.5, size).astype(np.float32) for _ in range(3)]
    gam = [rng.uniform(0.0, 0.2, size).astype(np.float32) for _ in range(3)]
    j0 = [(0.05 * rng.standard_normal(size)).astype(np.float32) for _ in range(3)]
    t = np.arange(20, dtype=np.float64)
    c = tuple(n // 2 for n in shape)
    sources = [("ez", c, F.gaussian_sine(t, 3.0, 2.0, 0.1)),
               ("ex", (origin[0] + 1, origin[1] + 1, origin[2] + 1), F.gaussian_sine(t, 4.0, 2.0, 0.1))]
    return ce, init, wp, gam, j0, sources


def _oracle(shape, npml, origin, ce, init, wp, gam, j0, sources, nsteps):
    cja, cjb = zip(*[oracle.drude_coefficients(w, g) for w, g in zip(wp, gam)])
    fields = {k: init[k].copy() for k in NAMES}
    fields.update(cex=ce[0], cey=ce[1], cez=ce[2])
    sim = oracle.OracleSim(fields, (npml,) * 3, 0x3F, _tables((npml,) * 3),
                           [(cc, ijk, a.astype(np.float32)) for cc, ijk, a in sources],
                           drude=(origin, [j.copy() for j in j0], list(cja), list(cjb)))
    sim.step(nsteps)
    return sim


@pytest.mark.parametrize("shape,npml,origin,size,tile", [
    ((40, 36, 70), 6, (10, 8, 20), (16, 14, 30), None),
    ((40, 36, 70), 6, (0, 0, 0), (40, 36, 70), (8, 16, 0, 3)),     # the whole grid, CPML inside the box
    ((33, 30, 45), 5, (3, 2, 1), (12, 20, 40), (4, 8, 0, 4)),      # box across z and y slabs, odd extents
    ((30, 44, 96), 4, (5, 7, 60), (9, 11, 36), (16, 8, 1, 3)),     # box at the back z face
])
def test_fused_and_unfused_step_with_drude_bit_exact(F, shape, npml, origin, size, tile):
    nsteps = 8
    ce, init, wp, gam, j0, sources = _case(F, shape, npml, origin, size, 31)
    sim = _oracle(shape, npml, origin, ce, init, wp, gam, j0, sources, nsteps)
    for fused in (True, False):
        d = F.DrudeAde(shape, origin, size)
        d.set_coeff(wp, gam)
        for q in range(3):
            d.J[q].copy_(torch.from_numpy(j0[q]))
        s = F.YeeSolver(shape, ce=ce, npml=npml, sources=sources, tile=tile, drude=d)
        s.set_fields(**init)
        if fused:
            s.step(nsteps)
        else:
            s.step_unfused(nsteps)
        torch.cuda.synchronize()
        s.check_status()
        tag = "fused" if fused else "unfused"
        for k in NAMES:
            np.testing.assert_array_equal(_host(s.fields[k]), sim.f[k], err_msg="%s %s" % (tag, k))
        for q in range(3):
            np.testing.assert_array_equal(_host(d.J[q]), sim.drude[1][q], err_msg="%s J%d" % (tag, q))
        for q in range(6):
            if s.psi_e()[q] is not None:
                np.testing.assert_array_equal(_host(s.psi_e()[q]), sim.psi_e[q], err_msg="%s psi_e%d" % (tag, q))
                np.testing.assert_array_equal(_host(s.cpml.psi_h[q]), sim.psi_h[q], err_msg="%s psi_h%d" % (tag, q))


def test_batched_grid_with_drude_equals_single(F):
    shapes = [((40, 36, 70), 6, (10, 8, 20), (16, 14, 30)), ((32, 32, 40), 4, None, None)]
    singles, batched, regions = [], [], []
    for n, (shape, npml, origin, size) in enumerate(shapes):
        ce, init, wp, gam, j0, sources = _case(F, shape, npml, origin or (1, 1, 1), size or (4, 4, 4), 40 + n)
        pair = []
        for _ in range(2):
            d = None
            if origin is not None:
                d = F.DrudeAde(shape, origin, size)
                d.set_coeff(wp, gam)
                for q in range(3):
                    d.J[q].copy_(torch.from_numpy(j0[q]))
            s = F.YeeSolver(shape, ce=ce, npml=npml, sources=sources, drude=d)
            s.set_fields(**init)
            pair.append((s, d))
        singles.append(pair[0])
        batched.append(pair[1])
    batch = F.BatchSolver([s for s, _ in batched])
    for s, _ in singles:
        s.step(6)
    batch.step(6)
    torch.cuda.synchronize()
    batch.check_status()
    for (a, da), (b, db) in zip(singles, batched):
        for k in NAMES:
            assert torch.equal(a.fields[k], b.fields[k]), k
        if da is not None:
            assert torch.equal(da.J, db.J)


def test_drude_argument_errors(F):
    with pytest.raises(ValueError):
        F.DrudeAde((10, 10, 10), (5, 5, 5), (6, 2, 2))
    d = F.DrudeAde((10, 10, 10), (1, 1, 1), (2, 2, 2))
    with pytest.raises(ValueError):
        F.YeeSolver((12, 10, 10), drude=d)

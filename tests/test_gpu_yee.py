"""GPU parity of the 2nd-order Yee kernels against the oracle and the
reference's golden outputs (bit-exact: the kernels evaluate the reference's
FP32 expressions with the same rounding and no FMA contraction)."""
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
def fdtd():
    import fdtd_accelerate_gb300 as F
    F.build()
    return F


def _dev(a, pad=0):
    """Device copy; pad > 0 gives a z-padded view with the same logical shape."""
    nx, ny, nz = a.shape
    if pad == 0:
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()
    store = torch.zeros((nx, ny, nz + pad), dtype=torch.float32, device="cuda")
    v = store[:, :, :nz]
    v.copy_(torch.from_numpy(a))
    return v


def _host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("shape,pad", [((9, 8, 12), 0), ((17, 19, 23), 0), ((17, 19, 23), 5),
                                       ((2, 3, 4), 0), ((64, 33, 130), 2)])
def test_update_e_h_bit_exact_vs_oracle(fdtd, shape, pad):
    rng = np.random.default_rng(7)
    h = {k: rng.standard_normal(shape).astype(np.float32) for k in NAMES}
    ce = [rng.random(shape, dtype=np.float32) for _ in range(3)]
    ch = [rng.random(shape, dtype=np.float32) for _ in range(3)]
    d = {k: _dev(v, pad) for k, v in h.items()}
    dce = [_dev(c, pad) for c in ce]
    dch = [_dev(c, pad) for c in ch]
    for step in range(3):
        oracle.update_e(*(h[k] for k in NAMES), *ce)
        fdtd.update_e(*(d[k] for k in NAMES), *dce)
        if step == 1:
            oracle.update_h(*(h[k] for k in NAMES), *ch)
            fdtd.update_h(*(d[k] for k in NAMES), *dch)
        else:
            oracle.update_h(*(h[k] for k in NAMES))
            fdtd.update_h(*(d[k] for k in NAMES))
    torch.cuda.synchronize()
    for k in NAMES:
        np.testing.assert_array_equal(_host(d[k]), h[k], err_msg=k)


def test_golden_numpy_reference_through_gpu(fdtd, golden_dir):
    """Reference fdtd3d.py outputs (tests/golden/yee_numpy.npz) reproduced by
    the GPU kernels called through the reference-shaped API."""
    g = np.load(os.path.join(golden_dir, "yee_numpy.npz"))
    for n in range(int(g["ncases"])):
        t = "c%d_" % n
        d = {k: _dev(g[t + "in_" + k]) for k in NAMES}
        ce = [_dev(g[t + "in_" + k]) for k in ("cex", "cey", "cez")]
        nsteps, axes = (int(v) for v in g[t + "meta"])
        src = tuple(int(v) for v in g[t + "src"])
        dirs = "".join(a for b, a in ((1, "x"), (2, "y"), (4, "z")) if axes & b)
        for s in range(nsteps):
            fdtd.update_e(*(d[k] for k in NAMES), *ce)
            if dirs:
                fdtd.update_pbc_e(dirs, d["ex"], d["ey"], d["ez"])
            d["ez"][src] += float(g[t + "amps"][s])
            fdtd.update_h(*(d[k] for k in NAMES))
            if dirs:
                fdtd.update_pbc_h(dirs, d["hx"], d["hy"], d["hz"])
        for k in NAMES:
            np.testing.assert_array_equal(_host(d[k]), g[t + "out_" + k], err_msg="case %d %s" % (n, k))


def test_golden_kemp_core_through_gpu(fdtd, golden_dir):
    """KEMP's SSE core groups the curl differently: agreement to 4 ulp."""
    g = np.load(os.path.join(golden_dir, "kemp_core.npz"))
    for n in range(int(g["ncases"])):
        t = "c%d_" % n
        nz, pad, coeff, ufunc = (int(v) for v in g[t + "meta"])
        d = {k: _dev(g[t + "in_" + k], pad) for k in NAMES}
        if ufunc == 0:
            fdtd.update_e(*(d[k] for k in NAMES), *(_dev(g[t + "in_" + k], pad) for k in ("cex", "cey", "cez")))
            comps = NAMES[:3]
        else:
            ch = [_dev(g[t + "in_" + k], pad) for k in ("chx", "chy", "chz")] if coeff else [None] * 3
            fdtd.update_h(*(d[k] for k in NAMES), *ch)
            comps = NAMES[3:]
        for k in comps:
            ref = g[t + "out_" + k]
            tol = 4 * np.finfo(np.float32).eps * max(1.0, np.abs(ref).max())
            assert np.abs(_host(d[k]) - ref).max() <= tol, (n, k)


def _kappa_tables(npml):
    t = [oracle.cpml_tables(p) for p in npml]
    return {key: [t[a][key] if npml[a] else None for a in range(3)]
            for key in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}


@pytest.mark.parametrize("shape,npml,faces", [((20, 18, 22), (3, 4, 5), 0x3F), ((20, 18, 22), (3, 0, 5), 0x15),
                                              ((31, 27, 16), (6, 6, 6), 0x2A)])
def test_cpml_kernels_bit_exact_vs_oracle(fdtd, shape, npml, faces):
    rng = np.random.default_rng(3)
    f = {k: rng.standard_normal(shape).astype(np.float32) for k in NAMES}
    ce = [rng.random(shape, dtype=np.float32) for _ in range(3)]
    layer = fdtd.CpmlLayer(shape, npml, faces)
    # the device layer's FP32 tables are the oracle's FP64 tables rounded once
    tables = _kappa_tables(layer.npml)
    for key in tables:
        for a in range(3):
            if layer.npml[a]:
                np.testing.assert_array_equal(layer.tables[a][key].cpu().numpy(),
                                              tables[key][a].astype(np.float32))
    P = layer.npml
    pshape = [(2 * P[0], shape[1], shape[2]), (shape[0], 2 * P[1], shape[2]), (shape[0], shape[1], 2 * P[2])]
    psi_e = [np.zeros(pshape[a], np.float32) if P[a] else None for a in range(3) for _ in range(2)]
    psi_h = [np.zeros(pshape[a], np.float32) if P[a] else None for a in range(3) for _ in range(2)]
    d = {k: _dev(v) for k, v in f.items()}
    dce = [_dev(c) for c in ce]
    for _ in range(4):
        oracle.update_e(*(f[k] for k in NAMES), *ce)
        oracle.cpml_e(P, layer.faces, tables, *(f[k] for k in NAMES), *ce, psi_e)
        oracle.update_h(*(f[k] for k in NAMES))
        oracle.cpml_h(P, layer.faces, tables, *(f[k] for k in NAMES), psi_h)
        fdtd.update_e(*(d[k] for k in NAMES), *dce)
        layer.update_e(*(d[k] for k in NAMES), *dce)
        fdtd.update_h(*(d[k] for k in NAMES))
        layer.update_h(*(d[k] for k in NAMES))
    torch.cuda.synchronize()
    for k in NAMES:
        np.testing.assert_array_equal(_host(d[k]), f[k], err_msg=k)
    for q in range(6):
        if psi_e[q] is not None:
            np.testing.assert_array_equal(_host(layer.psi_e[0][q]), psi_e[q], err_msg="psi_e%d" % q)
            np.testing.assert_array_equal(_host(layer.psi_h[q]), psi_h[q], err_msg="psi_h%d" % q)


def _oracle_sim(work_shape, ce, npml, faces, sources, init):
    tables = _kappa_tables(npml)
    fields = {k: init[k].copy() for k in NAMES}
    fields.update(cex=ce[0], cey=ce[1], cez=ce[2])
    return oracle.OracleSim(fields, npml, faces, tables,
                            [(c, ijk, a.astype(np.float32)) for c, ijk, a in sources])


@pytest.mark.parametrize("shape,npml,tile", [
    ((37, 29, 45), 5, None),
    ((37, 29, 45), 5, (4, 7, 0, 6)),
    ((40, 33, 64), 6, (16, 16, 0, 3)),
    ((24, 20, 36), 0, (8, 5, 0, 3)),
    ((70, 9, 100), 3, (8, 64, 0, 4)),
    ((41, 35, 70), 4, (16, 8, 1, 3)),    # persistent: many work items per CTA
    ((41, 35, 70), 4, (8, 3, 1, 3)),
    ((19, 66, 33), 4, (16, 2, 1, 3)),
    ((40, 40, 200), 4, (8, 16, 0, 4)),   # interior tiles take the packed fast path
    ((30, 44, 260), 3, None),
    ((24, 40, 200), 0, (4, 8, 0, 4)),
    ((37, 29, 45), 5, (8, 16, 0, 3, 2)),      # L2 promotion variants
    ((40, 40, 200), 4, (8, 16, 0, 4, 1)),
    ((30, 44, 70), 14, (16, 8, 1, 3)),        # z band wider than half a tile
    ((30, 44, 72), 14, (16, 8, 1, 3)),        # TMA band kernels, 16-wide boxes at their limit
    ((36, 36, 96), 16, None),                 # TMA band kernels, 32-wide boxes
    ((33, 21, 64), 6, (8, 16, 0, 3)),         # TMA band kernels, ragged y tiles
    ((24, 20, 192), 5, None),                 # three z tiles, sources in the middle one
])
def test_fused_step_bit_exact_vs_oracle_and_unfused(fdtd, shape, npml, tile):
    from fdtd_accelerate_gb300 import configs
    rng = np.random.default_rng(11)
    spheres = configs.random_spheres(rng, shape, 6, 2, 6, 1.0, 12.0)
    ce = [c.numpy() for c in configs.ce_from_spheres(shape, spheres)]
    nsteps = 9
    t = np.arange(nsteps + 2, dtype=np.float64)
    sources = [("ez", (shape[0] // 2, shape[1] // 2, shape[2] // 2), fdtd.gaussian_sine(t, 3.0, 2.0, 0.1)),
               ("ex", (npml + 2, shape[1] - npml - 3, npml + 2), fdtd.gaussian_sine(t, 5.0, 2.0, 0.1)),
               ("ey", (shape[0] // 3, 1, shape[2] - 2), fdtd.gaussian_sine(t, 4.0, 3.0, 0.1))]
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    faces = 0x3F
    sim = _oracle_sim(shape, ce, (npml,) * 3, faces, sources, init)
    sim.step(nsteps)

    fused = fdtd.YeeSolver(shape, ce=ce, npml=npml, faces=faces, sources=sources, tile=tile)
    fused.set_fields(**init)
    fused.step(nsteps)
    unf = fdtd.YeeSolver(shape, ce=ce, npml=npml, faces=faces, sources=sources)
    unf.set_fields(**init)
    unf.step_unfused(nsteps)
    torch.cuda.synchronize()
    fused.check_status()
    for k in NAMES:
        np.testing.assert_array_equal(_host(unf.fields[k]), sim.f[k], err_msg="unfused " + k)
        np.testing.assert_array_equal(_host(fused.fields[k]), sim.f[k], err_msg="fused " + k)
    if npml:
        for q in range(6):
            np.testing.assert_array_equal(_host(fused.psi_e()[q]), sim.psi_e[q], err_msg="psi_e%d" % q)
            np.testing.assert_array_equal(_host(fused.cpml.psi_h[q]), sim.psi_h[q], err_msg="psi_h%d" % q)


@pytest.mark.parametrize("shape,npml,faces,tile", [
    ((30, 26, 90), 6, 0x10, None),            # z front face only
    ((30, 26, 90), 6, 0x20, (8, 16, 0, 3)),   # z back face only
    ((30, 26, 90), 6, 0x33, (4, 8, 0, 4)),    # x and z faces, 4-row tiles
    ((26, 30, 60), 8, 0x3F, (16, 8, 1, 3)),   # one z tile holds both z slabs
    ((30, 26, 90), 7, 0x30, None),            # odd slab width
    ((20, 18, 192), 8, 0x3F, None),           # three z tiles
    ((20, 18, 256), 6, 0x20, (8, 16, 0, 3)),  # back face only, four z tiles
    ((20, 18, 140), 6, 0x3F, (4, 8, 0, 4)),   # short last z tile
    ((20, 18, 135), 6, 0x3F, None),           # last z tile of 7 cells, all of them in the H band
])
def test_fused_z_slab_faces_and_sources(fdtd, shape, npml, faces, tile):
    """The z-slab CPML (band kernels after the fused kernel) with one or both z
    faces, and soft sources of every component on E z-slab nodes of both sides
    (two of them on one cell: list order; some on the rows next to a tile edge
    in y), equals the oracle bit for bit."""
    rng = np.random.default_rng(23)
    ce = [(0.5 / rng.uniform(1.0, 6.0, shape)).astype(np.float32) for _ in range(3)]
    nsteps = 7
    t = np.arange(nsteps + 2, dtype=np.float64)
    nz = shape[2]
    sources = []
    for n, (comp, k) in enumerate([("ex", 1), ("ey", npml), ("ez", 2), ("ex", nz - npml - 1), ("ey", nz - 2),
                                   ("ez", nz - 3), ("ex", 1)]):
        sources.append((comp, (shape[0] // 2 + n % 3, shape[1] // 2 - n % 2, k), fdtd.gaussian_sine(t, 2.0 + n, 2.0, 0.1)))
    for n, (comp, j, k) in enumerate([("ex", 8, 1), ("ey", 7, nz - 2), ("ez", 4, npml), ("ey", 3, nz - npml - 1)]):
        sources.append((comp, (shape[0] // 3, j, k), fdtd.gaussian_sine(t, 3.0 + n, 2.0, 0.1)))
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    sim = _oracle_sim(shape, ce, (npml,) * 3, faces, sources, init)
    sim.step(nsteps)
    fused = fdtd.YeeSolver(shape, ce=ce, npml=npml, faces=faces, sources=sources, tile=tile)
    fused.set_fields(**init)
    assert fused.plan_info()["z_band"] == 1
    assert fused.plan_info()["launches_per_step"] == 3
    fused.step(nsteps)
    torch.cuda.synchronize()
    fused.check_status()
    for k in NAMES:
        np.testing.assert_array_equal(_host(fused.fields[k]), sim.f[k], err_msg=k)
    for q in range(6):
        if fused.psi_e()[q] is not None:  # axes without a CPML face have no slabs
            np.testing.assert_array_equal(_host(fused.psi_e()[q]), sim.psi_e[q], err_msg="psi_e%d" % q)
            np.testing.assert_array_equal(_host(fused.cpml.psi_h[q]), sim.psi_h[q], err_msg="psi_h%d" % q)


@pytest.mark.parametrize("tile", [None, (8, 16, 0, 3)])
def test_fused_line_source_many_per_tile(fdtd, tile):
    """A z line of 90 sources (a tile holds up to 65 of them, plus a second
    line crossing the same tiles in y) equals the oracle; a layout with more
    sources in one tile than the kernel can hold is refused at plan time."""
    shape, npml = (30, 34, 100), 4
    rng = np.random.default_rng(2)
    t = np.arange(12, dtype=np.float64)
    amp = fdtd.gaussian_sine(t, 3.0, 2.0, 0.1)
    sources = [("ez", (7, 17, k), amp * (1 + 0.01 * k)) for k in range(5, 95)]
    sources += [("ex", (12, j, 40), amp) for j in range(5, 29)]
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    ce = [np.full(shape, 0.5, np.float32) for _ in range(3)]
    sim = _oracle_sim(shape, ce, (npml,) * 3, 0x3F, sources, init)
    sim.step(8)
    fused = fdtd.YeeSolver(shape, ce=ce, npml=npml, sources=sources, tile=tile)
    fused.set_fields(**init)
    fused.step(8)
    torch.cuda.synchronize()
    fused.check_status()
    for k in NAMES:
        np.testing.assert_array_equal(_host(fused.fields[k]), sim.f[k], err_msg=k)
    crowded = [("ez", (7, 17, k), amp) for k in range(5, 95)] * 3   # 177 in the first z tile
    with pytest.raises(ValueError):
        fdtd.YeeSolver(shape, npml=npml, sources=crowded).plan()


def test_fused_then_unfused_interleave(fdtd):
    shape = (33, 30, 40)
    rng = np.random.default_rng(5)
    init = {k: rng.standard_normal(shape).astype(np.float32) for k in NAMES}
    a = fdtd.YeeSolver(shape, npml=4)
    b = fdtd.YeeSolver(shape, npml=4)
    a.set_fields(**init)
    b.set_fields(**init)
    a.step(3)
    a.step_unfused(2)
    a.step(2)
    b.step_unfused(7)
    torch.cuda.synchronize()
    for k in NAMES:
        np.testing.assert_array_equal(_host(a.fields[k]), _host(b.fields[k]), err_msg=k)


def test_bounded_wait_expires_and_solver_recovers(fdtd):
    """A pipeline wait that runs out: CTA 0 withholds the copies of one plane
    (nothing is in flight for it), its wait gives up after the shortened limit,
    the kernel records FDTD_ERR_TIMEOUT and returns; the context and the plan
    stay usable, and with the hook cleared the same plan steps bit-exactly."""
    import time
    shape, npml = (37, 29, 45), 5
    rng = np.random.default_rng(23)
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    t = np.arange(8, dtype=np.float64)
    sources = [("ez", (18, 14, 22), fdtd.gaussian_sine(t, 3.0, 2.0, 0.1))]
    a = fdtd.YeeSolver(shape, npml=npml, sources=sources)
    a.set_fields(**init)
    a.test_timeout(wait_ns=20_000_000, withhold_plane=1)   # 20 ms limit
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    a.step(1)
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(TimeoutError):
        a.check_status()
    assert int(a.status.item()) == 0   # check_status cleared the word

    # same plan, hook cleared, state reset: bit-exact against a fresh solver
    a.test_timeout()
    a.cpml.reset()
    a.cur, a.tstep = 0, 1
    a.set_fields(**init)
    b = fdtd.YeeSolver(shape, npml=npml, sources=sources)
    b.set_fields(**init)
    a.step(4)
    b.step(4)
    torch.cuda.synchronize()
    a.check_status()
    b.check_status()
    for k in NAMES:
        np.testing.assert_array_equal(_host(a.fields[k]), _host(b.fields[k]), err_msg=k)


def test_api_errors(fdtd):
    a = torch.zeros((4, 5, 6), device="cuda")
    with pytest.raises(TypeError):
        fdtd.update_h(a, a, a, a, a, a.double())
    with pytest.raises(TypeError):
        fdtd.update_e(a, a, a, a, a, a, a, a, np.zeros((4, 5, 6), np.float32))
    with pytest.raises(ValueError):
        fdtd.update_h(a, a, a, a, a, torch.zeros((4, 5, 7), device="cuda"))
    with pytest.raises(ValueError):
        fdtd.update_h(a, a, a, a, a, a.cpu())
    with pytest.raises(ValueError):
        fdtd.update_pbc_e("xw", a, a, a)
    with pytest.raises(ValueError):
        fdtd.YeeSolver((10, 10, 10), npml=5)   # 2P+2 > n


def test_cpml_absorbs_outgoing_pulse(fdtd):
    """A zero-mean pulse radiated from the centre leaves a CPML box: the field
    energy that remains is a small fraction of the PEC box's (lossless) energy."""
    shape = (64, 64, 64)
    t = np.arange(402, dtype=np.float64)
    amp = -(t - 30.0) / 36.0 * np.exp(-0.5 * ((t - 30.0) / 6.0) ** 2)
    energies = {}
    for npml in (0, 10):
        s = fdtd.YeeSolver(shape, npml=npml, sources=[("ez", (32, 32, 32), amp)])
        s.step(400)
        torch.cuda.synchronize()
        s.check_status()
        energies[npml] = sum(float((v.double() ** 2).sum()) for v in s.fields.values())
        assert np.isfinite(energies[npml])
    assert energies[10] < 0.01 * energies[0], energies

"""Batched fused step: every grid of a ragged batch equals its own single-grid
run bit for bit (fields and CPML psi), through plain launches, a captured
CUDA graph and autotuned launch shapes."""
import numpy as np
import pytest
import torch

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")

# (shape, npml, faces) of a small ragged batch: CPML on all or some faces,
# PEC-only grids, odd extents, one grid smaller than a tile
GRIDS = [((48, 32, 64), 8, 0x3F), ((32, 48, 32), 8, 0x3F), ((37, 29, 45), 5, 0x15),
         ((16, 12, 20), 0, 0x3F), ((64, 40, 96), 8, 0x2A), ((20, 70, 36), 4, 0x3F)]


@pytest.fixture(scope="module")
def F():
    import fdtd_accelerate_gb300 as F
    F.build()
    return F


def make_pair(F, seed, shape, npml, faces, nsteps=40):
    """Two identical grids (random spheres, a source, random initial fields)."""
    from fdtd_accelerate_gb300 import configs
    rng = np.random.default_rng(seed)
    sph = configs.random_spheres(rng, shape, 4, 2, max(2, min(shape) // 5), 1.0, 8.0)
    ce = configs.ce_from_spheres(shape, sph)
    t = np.arange(nsteps + 2, dtype=np.float64)
    src = [("ez", tuple(n // 2 for n in shape), np.sin(0.2 * t)),
           ("ex", (shape[0] // 3, shape[1] // 2, shape[2] // 3), np.cos(0.1 * t))]
    init = {k: rng.standard_normal(shape).astype(np.float32) * np.float32(0.1) for k in NAMES}
    out = []
    for _ in range(2):
        s = F.YeeSolver(shape, ce=ce, npml=npml, faces=faces, sources=src)
        s.set_fields(**init)
        out.append(s)
    return out


def assert_same(a, b, tag):
    fa, fb = a.fields, b.fields
    for k in NAMES:
        assert torch.equal(fa[k], fb[k]), "%s %s" % (tag, k)
    for q in range(6):
        pa, pb = a.cpml.psi_e[a.cur][q], b.cpml.psi_e[b.cur][q]
        if pa is not None:
            assert torch.equal(pa, pb), "%s psi_e%d" % (tag, q)
            assert torch.equal(a.cpml.psi_h[q], b.cpml.psi_h[q]), "%s psi_h%d" % (tag, q)


def build(F, tile=None, grids=GRIDS):
    singles, batched = [], []
    for n, (shape, npml, faces) in enumerate(grids):
        a, b = make_pair(F, 100 + n, shape, npml, faces)
        singles.append(a)
        batched.append(b)
    return singles, F.BatchSolver(batched, tile=tile)


@pytest.mark.parametrize("tile", [None, (8, 16, 0, 3), (4, 8, 0, 4), (16, 32, 1, 3), (8, 5, 2, 4)])
def test_batch_bit_identical_to_single(F, tile):
    singles, batch = build(F, tile)
    for s in singles:
        s.step(7)
    batch.step(3)
    batch.step(4)
    torch.cuda.synchronize()
    batch.check_status()
    for n, (a, b) in enumerate(zip(singles, batch.solvers)):
        assert a.tstep == b.tstep and a.cur == b.cur
        assert_same(a, b, "grid %d" % n)
    info = batch.plan_info()
    assert info["ctas"] >= 1 and info["items"] >= len(GRIDS)


def test_batch_graph_replay(F):
    singles, batch = build(F)
    for s in singles:
        s.step(6)
    batch.run_graph(6)
    torch.cuda.synchronize()
    for n, (a, b) in enumerate(zip(singles, batch.solvers)):
        assert_same(a, b, "graph grid %d" % n)
    # continue with plain launches after the graph
    for s in singles:
        s.step(3)
    batch.step(3)
    torch.cuda.synchronize()
    for n, (a, b) in enumerate(zip(singles, batch.solvers)):
        assert_same(a, b, "after graph grid %d" % n)


def test_batch_autotune_restores_state(F, tmp_path, monkeypatch):
    monkeypatch.setenv("FDTD_TUNE_CACHE", str(tmp_path / "tune.json"))
    singles, batch = build(F)
    entry = batch.autotune(candidates=((8, 64, 0, 3), (4, 32, 0, 4)), steps=2)
    assert tuple(entry["tile"]) in ((8, 64, 0, 3), (4, 32, 0, 4))
    assert (tmp_path / "tune.json").exists()
    for s in singles:
        s.step(5)
    batch.step(5)
    torch.cuda.synchronize()
    for n, (a, b) in enumerate(zip(singles, batch.solvers)):
        assert_same(a, b, "tuned grid %d" % n)
    # the second call reads the cache
    again = batch.autotune(candidates=((8, 64, 0, 3), (4, 32, 0, 4)), steps=2)
    assert again["tile"] == entry["tile"]


def test_batch_workload_shapes(F):
    from fdtd_accelerate_gb300 import configs
    works = configs.batched64(nsims=6, steps=4)
    batch = F.BatchSolver.from_workloads(works)
    batch.step(4)
    torch.cuda.synchronize()
    batch.check_status()
    singles = F.BatchSolver.from_workloads(works).solvers
    for s in singles:
        s.step(4)
    torch.cuda.synchronize()
    for n, (a, b) in enumerate(zip(singles, batch.solvers)):
        assert_same(a, b, "workload grid %d" % n)


def test_batch_argument_errors(F):
    import ctypes as C
    from fdtd_accelerate_gb300 import _native as N
    _, batch = build(F, grids=GRIDS[:2])
    L = N.lib()
    h = C.c_void_p()
    n = 2
    grids = (N.Grid * n)(*[s.grid() for s in batch.solvers])
    states = (N.YeeState * n)(*[s._state_struct() for s in batch.solvers])
    cpmls = (N.Cpml * n)(*[s.cpml.struct() for s in batch.solvers])
    srcs = (N.Sources * n)(*[s.sources.struct() for s in batch.solvers])
    tile = N.Tile(0, 0, 0, 0, 0)
    ws = batch.workspace
    status = C.c_void_p(batch.status.data_ptr())
    assert L.fdtd_batch_plan_create(C.byref(h), n, grids, states, cpmls, srcs, C.byref(tile), status,
                                    C.c_void_p(ws.data_ptr()), ws.numel() - 1, 0, None) == N.FDTD_ERR_CAPACITY
    assert L.fdtd_batch_plan_create(C.byref(h), n, grids, states, cpmls, srcs, C.byref(tile), status,
                                    C.c_void_p(ws.data_ptr() + 16), ws.numel(), 0, None) == N.FDTD_ERR_ALIGN
    assert L.fdtd_batch_plan_create(C.byref(h), 0, grids, states, cpmls, srcs, C.byref(tile), status,
                                    C.c_void_p(ws.data_ptr()), ws.numel(), 0, None) == N.FDTD_ERR_ARG
    with pytest.raises(ValueError):
        F.BatchSolver([])


def test_one_call_entry_points(F):
    """fdtd_yee_step_f32 and fdtd_batched_run_f32 (plan create, run and
    destroy in one call) give what the plans give, bit for bit, and report
    the buffer that holds the state afterwards."""
    import ctypes as C
    from fdtd_accelerate_gb300 import _native as N
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # single grid: 5 steps through the plan (a) and through one call (b)
    shape, npml, faces = GRIDS[2]
    a, b = make_pair(F, 7, shape, npml, faces)
    a.step(5)
    out = C.c_int32(-1)
    N.call("fdtd_yee_step_f32", C.byref(b.grid()), C.byref(b._state_struct()), C.byref(b.cpml.struct()),
           C.byref(b.sources.struct()), C.c_void_p(b.status.data_ptr()), b.cur, int(b.tstep), 5,
           C.byref(out), stream)
    torch.cuda.synchronize()
    assert out.value == a.cur
    b.cur, b.tstep = out.value, b.tstep + 5
    assert_same(a, b, "one-call step")
    # a batch: 4 steps through BatchSolver and through one call
    singles, batch = build(F)
    for s in singles:
        s.step(4)
    sv = batch.solvers
    n = len(sv)
    grids = (N.Grid * n)(*[s.grid() for s in sv])
    states = (N.YeeState * n)(*[s._state_struct() for s in sv])
    cpmls = (N.Cpml * n)(*[s.cpml.struct() for s in sv])
    srcs = (N.Sources * n)(*[s.sources.struct() for s in sv])
    out = C.c_int32(-1)
    N.call("fdtd_batched_run_f32", n, grids, states, cpmls, srcs, C.c_void_p(batch.status.data_ptr()),
           C.c_void_p(batch.workspace.data_ptr()), batch.workspace.numel(), sv[0].cur, int(sv[0].tstep), 4,
           C.byref(out), stream)
    torch.cuda.synchronize()
    for k, (s_single, s_batch) in enumerate(zip(singles, sv)):
        s_batch.cur, s_batch.tstep = out.value, s_batch.tstep + 4
        assert s_single.cur == out.value
        assert_same(s_single, s_batch, "one-call batch grid %d" % k)


def test_plan_creation_is_stream_ordered(F):
    """A batch plan created on a non-blocking stream, right after work on that
    stream rewrote a source position and with no device-wide synchronisation
    in between, sees the new position.  The source sits on an E z-slab node,
    which the batched band kernel takes from the host-side list that plan
    creation reads, so a read that ran ahead of the stream would drop it."""
    shape, npml, nsteps = (40, 36, 48), 6, 12
    t = np.arange(nsteps + 2, dtype=np.float64)
    good = (shape[0] // 2, shape[1] // 2, 1)                 # E z-slab node (front z face)
    src = [("ey", good, np.sin(0.3 * t))]
    rng = np.random.default_rng(9)
    init = {k: rng.standard_normal(shape).astype(np.float32) * np.float32(0.1) for k in NAMES}
    single = F.YeeSolver(shape, npml=npml, sources=src)
    single.set_fields(**init)
    other = F.YeeSolver(shape, npml=npml, sources=src)
    other.set_fields(**init)
    batch = F.BatchSolver([other])
    right = other.sources.ijk.clone()
    other.sources.ijk.copy_(torch.tensor([good[0], good[1], shape[2] // 2], dtype=torch.int32, device="cuda"))
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        torch.cuda._sleep(200_000_000)          # keep the stream busy well past the plan call
        other.sources.ijk.copy_(right)          # the position the plan must see
        batch.plan()
        batch.step(nsteps)
    single.step(nsteps)
    torch.cuda.synchronize()
    batch.check_status()
    assert_same(single, other, "stream-ordered plan")

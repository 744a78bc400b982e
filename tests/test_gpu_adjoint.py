"""Adjoint (reverse-time) kernels and the differentiable run.

* one adjoint step equals FP64 autograd of one forward step (the transpose of
  the E/H/CPML map and the dL/dCE term), on random states;
* the checkpointed run's forward equals YeeSolver bit for bit, and its
  gradient does not depend on the checkpoint interval;
* dL/dCE of a whole run agrees with FP64 autograd through the restated step
  (oracle/torch_ref.py) and with central finite differences."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from oracle.torch_ref import TorchYee
from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


@pytest.fixture(scope="module")
def F():
    import fdtd_accelerate_gb300 as F
    F.build()
    return F


def e_mask(shape, q):
    nx, ny, nz = shape
    m = np.zeros(shape, bool)
    if q == 0:
        m[:, :ny - 1, :nz - 1] = True
    elif q == 1:
        m[:nx - 1, :, :nz - 1] = True
    else:
        m[:nx - 1, :ny - 1, :] = True
    return m


def h_mask(shape, q):
    m = np.zeros(shape, bool)
    if q == 0:
        m[:, 1:, 1:] = True
    elif q == 1:
        m[1:, :, 1:] = True
    else:
        m[1:, 1:, :] = True
    return m


def rel_err(a, b, mask=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    scale = max(np.abs(b).max(), 1e-30)
    return np.abs(a - b).max() / scale


@pytest.mark.parametrize("shape,npml,faces", [((20, 18, 22), 4, 0x3F), ((17, 21, 19), 3, 0x19),
                                              ((16, 16, 16), 0, 0x3F)])
def test_adjoint_step_is_transpose(F, shape, npml, faces):
    from fdtd_accelerate_gb300 import _native as N
    from fdtd_accelerate_gb300.cpml import CpmlLayer
    rng = np.random.default_rng(11)
    layer = CpmlLayer(shape, npml, faces)
    P = layer.npml
    tabs = [{k: v.double().cpu() for k, v in t.items()} if p else None for t, p in zip(layer.tables, P)]
    ref = TorchYee(shape, P, layer.faces, tabs)
    E0, H0, pe0, ph0 = ref.zero_state()
    f32 = lambda s: torch.from_numpy(rng.standard_normal(s).astype(np.float32)).double()
    E = [f32(shape).requires_grad_(True) for _ in range(3)]
    H = [f32(shape).requires_grad_(True) for _ in range(3)]
    pe = [f32(p.shape).requires_grad_(True) if p is not None else None for p in pe0]
    ph = [f32(p.shape).requires_grad_(True) if p is not None else None for p in ph0]
    ce = [torch.from_numpy((0.5 / (1 + 7 * rng.random(shape))).astype(np.float32)).double().requires_grad_(True)
          for _ in range(3)]
    E1, H1, pe1, ph1 = ref.step(E, H, pe, ph, ce)
    lam_f = [f32(shape) for _ in range(6)]
    lam_pe = [f32(p.shape) if p is not None else None for p in pe0]
    lam_ph = [f32(p.shape) if p is not None else None for p in ph0]
    L = sum((a * b).sum() for a, b in zip(E1 + H1, lam_f))
    for a, b in zip(pe1 + ph1, lam_pe + lam_ph):
        if a is not None:
            L = L + (a * b).sum()
    L.backward()

    dev = torch.device("cuda")
    cu = lambda t: t.detach().float().contiguous().to(dev)
    lf = [cu(t) for t in lam_f]
    lpe = [cu(t) if t is not None else None for t in lam_pe]
    lph = [cu(t) if t is not None else None for t in lam_ph]
    we = [torch.zeros_like(t) if t is not None else None for t in lpe]
    wh = [torch.zeros_like(t) if t is not None else None for t in lph]
    gce = [torch.zeros(shape, device=dev) for _ in range(3)]
    hp = [cu(t) for t in H]
    pcur = [cu(t) if t is not None else None for t in pe1]
    cec = [cu(t) for t in ce]
    st = N.AdjointState()
    ptr = lambda t: t.data_ptr() if t is not None else None
    for q in range(6):
        st.lf[q] = ptr(lf[q])
        st.lpsi_e[q], st.lpsi_h[q], st.w_e[q], st.w_h[q] = ptr(lpe[q]), ptr(lph[q]), ptr(we[q]), ptr(wh[q])
    for q in range(3):
        st.grad_ce[q] = ptr(gce[q])
    nx, ny, nz = shape
    g = N.Grid(nx, ny, nz, ny * nz, nz)
    cp = layer.struct()
    N.call("fdtd_adjoint_step_f32", C.byref(g), C.byref(cp), C.byref(st), (C.c_void_p * 3)(*map(ptr, hp)),
           (C.c_void_p * 6)(*map(ptr, pcur)), (C.c_void_p * 3)(*map(ptr, cec)), None, None,
           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    for q in range(3):
        assert rel_err(lf[q].cpu(), E[q].grad, e_mask(shape, q)) < 2e-6, "lambda %s" % NAMES[q]
        assert rel_err(lf[3 + q].cpu(), H[q].grad, h_mask(shape, q)) < 2e-6, "lambda %s" % NAMES[3 + q]
        assert rel_err(gce[q].cpu(), ce[q].grad) < 2e-6, "dL/dce%d" % q
    for q in range(6):
        if pe[q] is not None:
            assert rel_err(lpe[q].cpu(), pe[q].grad) < 2e-6, "lambda psi_e%d" % q
            assert rel_err(lph[q].cpu(), ph[q].grad) < 2e-6, "lambda psi_h%d" % q


def make_case(shape, npml, nsteps, seed=3):
    """CE from random spheres, one Ez source, Ez/Ex monitors."""
    from fdtd_accelerate_gb300 import configs
    rng = np.random.default_rng(seed)
    sph = configs.random_spheres(rng, shape, 4, 2, max(2, min(shape) // 5), 1.0, 8.0)
    ce = torch.stack(configs.ce_from_spheres(shape, sph))
    t = np.arange(nsteps + 2, dtype=np.float64)
    amp = np.sin(2 * np.pi * 0.05 * t) * np.exp(-0.5 * ((t - 30.0) / 10.0) ** 2)
    src = [("ez", (shape[0] // 3, shape[1] // 2, shape[2] // 2), amp)]
    mons = [("ez", (2 * shape[0] // 3, shape[1] // 2, shape[2] // 2)),
            ("ex", (2 * shape[0] // 3, shape[1] // 2 + 2, shape[2] // 2 - 1)),
            ("hy", (shape[0] // 2, shape[1] // 3, shape[2] // 2))]
    return ce, src, mons


def test_run_forward_matches_solver_and_segments(F):
    shape, npml, nsteps = (28, 24, 32), 5, 37
    ce, src, mons = make_case(shape, npml, nsteps)
    eng = F.YeeAdjoint(shape, nsteps, npml=npml, sources=src, monitors=mons, segment=10)
    cg = ce.cuda().requires_grad_(True)
    mon, final = F.fdtd_run(cg, eng)
    s = F.YeeSolver(shape, ce=ce, npml=npml, sources=src)
    rows = []
    for _ in range(nsteps):
        s.step(1)
        f = s.fields
        rows.append(torch.stack([f[c][p] for c, p in mons]))
    torch.cuda.synchronize()
    assert torch.equal(mon, torch.stack(rows))
    for q, k in enumerate(NAMES):
        assert torch.equal(final[q], s.fields[k]), k
    loss = (mon.double() ** 2).sum()
    (g1,) = torch.autograd.grad(loss, cg)
    eng2 = F.YeeAdjoint(shape, nsteps, npml=npml, sources=src, monitors=mons, segment=7)
    cg2 = ce.cuda().requires_grad_(True)
    mon2, _ = F.fdtd_run(cg2, eng2)
    (g2,) = torch.autograd.grad((mon2.double() ** 2).sum(), cg2)
    assert torch.equal(g1, g2)
    assert float(g1.abs().max()) > 0


def ref_grad(shape, npml, nsteps, ce, src, mons, faces=0x3F, every=20, dtype=torch.float64):
    """Monitors and dL/dCE from autograd through the restated step (the
    loss accumulated in FP64 either way)."""
    from fdtd_accelerate_gb300.cpml import CpmlLayer
    layer = CpmlLayer(shape, npml, faces, device="cpu")
    tabs = [{k: v.to(dtype) for k, v in t.items()} if p else None for t, p in zip(layer.tables, layer.npml)]
    ref = TorchYee(shape, layer.npml, layer.faces, tabs, dtype=dtype)
    cer = ce.to(dtype).clone().requires_grad_(True)
    srcs = [(NAMES.index(c), ijk, np.asarray(a, np.float32).astype(np.float64)) for c, ijk, a in src]
    mons_i = [(NAMES.index(c), ijk) for c, ijk in mons]
    mon, _ = ref.run(list(cer), nsteps, srcs, mons_i, checkpoint_every=every)
    (mon.double() ** 2).sum().backward()
    return mon.detach().double(), cer.grad.double()


@pytest.mark.parametrize("shape,npml,nsteps", [((24, 22, 26), 4, 80), ((64, 64, 64), 8, 60)])
def test_gradient_vs_fp64_autograd(F, shape, npml, nsteps):
    ce, src, mons = make_case(shape, npml, nsteps)
    eng = F.YeeAdjoint(shape, nsteps, npml=npml, sources=src, monitors=mons, segment=25)
    cg = ce.cuda().requires_grad_(True)
    mon, _ = F.fdtd_run(cg, eng)
    (mon.double() ** 2).sum().backward()
    mon_ref, g_ref = ref_grad(shape, npml, nsteps, ce, src, mons)
    assert rel_err(mon.detach().cpu(), mon_ref) < 1e-5
    # the FP32 floor: the same autograd run in FP32 against FP64
    _, g32 = ref_grad(shape, npml, nsteps, ce, src, mons, dtype=torch.float32)
    g = cg.grad.cpu()
    for q in range(3):
        err = rel_err(g[q], g_ref[q])
        floor = rel_err(g32[q], g_ref[q])
        print("dL/dce%d: adjoint %.2e, FP32 autograd %.2e (max-normalised vs FP64)" % (q, err, floor))
        assert err < max(1e-4, 3 * floor), "dL/dce%d relative error %.2e (FP32 floor %.2e)" % (q, err, floor)


def test_design_region_gradient_equals_full_gradient_inside(F):
    """grad_region (fdtd_adjoint_step_region_f32): inside the box the gradient
    equals the whole-grid run bit for bit (the adjoint fields do not depend on
    the box), outside it is zero; the box may touch the CPML slabs."""
    shape, npml, nsteps = (30, 28, 36), 5, 60
    ce, src, mons = make_case(shape, npml, nsteps, seed=4)
    region = (slice(3, 21), slice(7, 28), slice(0, 17))
    grads = []
    for reg in (None, region):
        eng = F.YeeAdjoint(shape, nsteps, npml=npml, sources=src, monitors=mons, segment=16, grad_region=reg)
        cg = ce.cuda().requires_grad_(True)
        mon, _ = F.fdtd_run(cg, eng)
        (mon.double() ** 2).sum().backward()
        grads.append(cg.grad.detach().cpu())
        eng.close()
    full, part = grads
    mask = torch.zeros(shape, dtype=torch.bool)
    mask[region] = True
    for q in range(3):
        np.testing.assert_array_equal(part[q][mask].numpy(), full[q][mask].numpy(), err_msg="dL/dce%d inside" % q)
        assert not part[q][~mask].any(), "dL/dce%d outside the region" % q
    assert full[:, ~mask].abs().max() > 0   # the whole-grid gradient is not zero there
    with pytest.raises(ValueError):
        F.YeeAdjoint(shape, nsteps, npml=npml, grad_region=(slice(0, 0), slice(None), slice(None)))


@pytest.mark.parametrize("region", [None, (slice(4, 20), slice(6, 22), slice(3, 30))])
def test_overlapped_backward_equals_serial(F, region):
    """overlap=True (segment c-1 recomputed into a second slot set on a side
    stream beside the reverse steps of segment c) gives the same gradient and
    monitor series bit for bit as the serial backward, over several segments
    (the last one ragged), twice in a row on the same engine."""
    shape, npml, nsteps = (26, 28, 34), 5, 47
    ce, src, mons = make_case(shape, npml, nsteps, seed=6)
    out = []
    for overlap in (False, True):
        eng = F.YeeAdjoint(shape, nsteps, npml=npml, sources=src, monitors=mons, segment=9,
                           grad_region=region, overlap=overlap)
        for _ in range(2):
            cg = ce.cuda().requires_grad_(True)
            mon, _ = F.fdtd_run(cg, eng)
            (mon.double() ** 2).sum().backward()
            out.append((mon.detach().cpu(), cg.grad.detach().cpu()))
        eng.check_status()
        eng.close()
    ref_mon, ref_g = out[0]
    for mon, g in out[1:]:
        np.testing.assert_array_equal(mon.numpy(), ref_mon.numpy())
        np.testing.assert_array_equal(g.numpy(), ref_g.numpy())
    assert ref_g.abs().max() > 0


def test_gradient_vs_finite_differences(F):
    """Central differences in eps (h = 1e-3) at cells near the monitors against
    dL/deps from the adjoint run with CE = 0.5/eps for all three components of
    a cell.  The differenced loss is evaluated in FP64 on the restated step
    (the exact loss of the FP32-rounded CE): two FP32 runs differ by roundoff
    of the order of the perturbation itself (g h / L ~ 1e-7..1e-5 here)."""
    from fdtd_accelerate_gb300.cpml import CpmlLayer
    shape, npml, nsteps = (32, 30, 34), 6, 150
    ce0, src, mons = make_case(shape, npml, nsteps, seed=9)
    eps0 = (0.5 / ce0[2]).double()
    eng = F.YeeAdjoint(shape, nsteps, npml=npml, sources=src, monitors=mons, segment=50)
    eps = eps0.cuda().requires_grad_(True)
    cef = (0.5 / eps).float().unsqueeze(0).expand(3, -1, -1, -1).contiguous()
    mon, _ = F.fdtd_run(cef, eng)
    (mon.double() ** 2).sum().backward()
    g = eps.grad.cpu()
    layer = CpmlLayer(shape, npml, 0x3F, device="cpu")
    ref = TorchYee(shape, layer.npml, layer.faces, [{k: v.double() for k, v in t.items()} for t in layer.tables])
    srcs = [(NAMES.index(c), ijk, np.asarray(a, np.float32).astype(np.float64)) for c, ijk, a in src]
    mons_i = [(NAMES.index(c), ijk) for c, ijk in mons]

    def loss64(e):
        ce = (0.5 / e.float()).double()
        m, _ = ref.run([ce, ce, ce], nsteps, srcs, mons_i)
        return float((m ** 2).sum())

    rng = np.random.default_rng(21)
    cells = []
    while len(cells) < 8:
        c = tuple(int(rng.integers(lo, hi)) for lo, hi in
                  ((shape[0] // 3, 2 * shape[0] // 3 + 2), (shape[1] // 2 - 3, shape[1] // 2 + 4),
                   (shape[2] // 2 - 3, shape[2] // 2 + 4)))
        if c not in cells:
            cells.append(c)
    h = 1e-3
    errs = []
    for c in cells:
        vals = []
        for sgn in (1, -1):
            e2 = eps0.clone()
            e2[c] += sgn * h
            vals.append(loss64(e2))
        fd = (vals[0] - vals[1]) / (2 * h)
        errs.append(abs(fd - float(g[c])) / max(abs(fd), 1e-30))
    print("FD relative errors", ["%.2e" % e for e in errs])
    assert max(errs) < 1e-3, errs


@pytest.mark.parametrize("n", [40, 1500])
def test_add_points_repeats_in_list_order(F, n):
    """fdtd_add_points_f32 equals a walk of the list in order (FP32 adds),
    with repeated (cell, component) pairs, one cell under several components
    and out-of-range points; 40 points take the one-thread-per-point kernel,
    1500 the list walk."""
    from fdtd_accelerate_gb300 import _native as N
    shape = (6, 5, 8)
    rng = np.random.default_rng(3 + n)
    f = [torch.tensor(rng.standard_normal(shape).astype(np.float32), device="cuda") for _ in range(6)]
    ijk = np.stack([rng.integers(0, s, n) for s in shape], axis=1).astype(np.int32)
    comp = rng.integers(0, 6, n).astype(np.int32)
    ijk[1::7] = ijk[0]                           # many repeats of one point, mixed components
    ijk[n // 2 + 1] = (9, 0, 0)                  # out of range: skipped
    vals = rng.standard_normal(n).astype(np.float32)
    want = [t.cpu().numpy().copy() for t in f]
    for p in range(n):
        i, j, k = ijk[p]
        if i < shape[0] and j < shape[1] and k < shape[2]:
            want[comp[p]][i, j, k] = np.float32(want[comp[p]][i, j, k] + vals[p])
    d_ijk = torch.tensor(ijk.ravel(), device="cuda")
    d_comp = torch.tensor(comp, device="cuda")
    d_vals = torch.tensor(vals, device="cuda")
    pts = N.Points(n, d_ijk.data_ptr(), d_comp.data_ptr())
    g = N.Grid(*shape, shape[1] * shape[2], shape[2])
    fp = (C.c_void_p * 6)(*[t.data_ptr() for t in f])
    rc = N.lib().fdtd_add_points_f32(C.byref(g), C.byref(pts), fp, C.c_void_p(d_vals.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    for q in range(6):
        np.testing.assert_array_equal(f[q].cpu().numpy(), want[q])

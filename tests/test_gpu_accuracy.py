"""Accuracy of the plain 128^3 workload (1000 steps, PEC, Ez source) at its
full size: the GPU equals the FP32 oracle (the reference's FP32 NumPy
arithmetic) bit for bit, and its distance to the FP64 oracle is the FP32
floor of that arithmetic.

Metric: max|a - b| over a component divided by the largest |b| of its field
family (E or H).  Per-component normalisation is meaningless for hz, which is
zero in exact arithmetic for an Ez source (its FP64 value is roundoff)."""
import numpy as np
import pytest
import torch

import oracle
from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


def oracle_run(work, dtype):
    f = {k: np.zeros(work.shape, dtype) for k in NAMES}
    for k in ("cex", "cey", "cez"):
        f[k] = np.full(work.shape, 0.5, dtype)
    srcs = [(c, ijk, a.astype(np.float32).astype(dtype)) for c, ijk, a in work.source_list()]
    sim = oracle.OracleSim(f, (0, 0, 0), 0x3F, None, srcs)
    sim.step(work.steps)
    return sim.f


def test_plain128_full_run_bit_exact_and_fp64_floor():
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    F.build()
    w = configs.plain128()
    s = F.YeeSolver(w.shape, sources=w.source_list())
    s.step(w.steps)
    torch.cuda.synchronize()
    s.check_status()
    gpu = {k: v.cpu().numpy() for k, v in s.fields.items()}
    f32 = oracle_run(w, np.float32)
    for k in NAMES:
        np.testing.assert_array_equal(gpu[k], f32[k], err_msg=k)
    f64 = oracle_run(w, np.float64)
    errs = {}
    for fam in (NAMES[:3], NAMES[3:]):
        scale = max(np.abs(f64[k]).max() for k in fam)
        for k in fam:
            errs[k] = np.abs(gpu[k].astype(np.float64) - f64[k]).max() / scale
    print("plain128, 1000 steps, FP32 vs FP64 (family-normalised):",
          ", ".join("%s %.2e" % (k, errs[k]) for k in NAMES))
    # the FP32 floor of the reference arithmetic; 1e-5 is not reachable bit-exactly
    assert max(errs.values()) < 1e-4, errs


def test_fp64_step_bit_exact_vs_fp64_oracle():
    """The GPU FP64 step (fdtd_step_unfused_f64) equals the FP64 C oracle bit for
    bit: CPML on all faces, a source, random initial state and coefficients."""
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300.fp64 import YeeRun64
    F.build()
    shape, npml, nsteps = (20, 18, 22), 4, 6
    rng = np.random.default_rng(17)
    ce = [(0.5 / (1 + 7 * rng.random(shape))) for _ in range(3)]
    t = np.arange(nsteps + 2, dtype=np.float64)
    src = [("ez", (10, 9, 11), np.sin(0.3 * t))]
    run = YeeRun64(shape, ce=ce, npml=npml, sources=src)
    init = {k: rng.standard_normal(shape) for k in NAMES}
    for q, k in enumerate(NAMES):
        run.f[q].copy_(torch.from_numpy(init[k]))
    run.step(nsteps)
    torch.cuda.synchronize()
    tabs = {k: [v[k].double().cpu().numpy() for v in run.cpml.tables] for k in run.cpml.tables[0]}
    fields = {k: init[k].copy() for k in NAMES}
    fields.update(cex=ce[0], cey=ce[1], cez=ce[2])
    amp = np.asarray(src[0][2], np.float32).astype(np.float64)
    sim = oracle.OracleSim(fields, (npml,) * 3, 0x3F, tabs, [("ez", (10, 9, 11), amp)])
    sim.step(nsteps)
    for q, k in enumerate(NAMES):
        np.testing.assert_array_equal(run.f[q].cpu().numpy(), sim.f[k], err_msg=k)
    for q in range(6):
        np.testing.assert_array_equal(run.psi_e[q].cpu().numpy(), sim.psi_e[q], err_msg="psi_e%d" % q)
        np.testing.assert_array_equal(run.psi_h[q].cpu().numpy(), sim.psi_h[q], err_msg="psi_h%d" % q)


def test_cpml1024_workload_fp32_vs_fp64_full_size():
    """The Yee + CPML workload at its own size (1024 x 1024 x 512, 12-cell CPML,
    200 spheres, 6 dipoles), 2000 steps: the fused FP32 path against the GPU
    FP64 step, same inputs (FP32 coefficients, tables and amplitudes widened).
    Per field family: max |a - b| / max |b| and the root-mean-square ratio."""
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    from fdtd_accelerate_gb300.fp64 import YeeRun64, family_errors
    F.build()
    work = configs.cpml1024(steps=2000)
    shape, nsteps = work.shape, work.steps
    ce = configs.ce_from_spheres(shape, work.spheres, device="cuda")
    src = work.source_list(nsteps + 2)
    s32 = F.YeeSolver(shape, ce=ce, npml=12, sources=src)
    s32.step(nsteps)
    s64 = YeeRun64(shape, ce=ce, npml=12, sources=src)
    del ce
    s64.step(nsteps)
    torch.cuda.synchronize()
    s32.check_status()
    errs = family_errors(s32.fields, s64.fields)
    print("cpml workload 1024x1024x512, %d steps, FP32 vs FP64 (family-normalised max / rms):" % nsteps,
          ", ".join("%s %.2e / %.2e" % (k, errs[k]["max"], errs[k]["rms"]) for k in NAMES))
    # The FP32 path equals the reference's FP32 arithmetic bit for bit; this is
    # that arithmetic's distance to FP64 at the workload's size and step count.
    assert max(e["max"] for e in errs.values()) < 3e-4, errs
    assert max(e["rms"] for e in errs.values()) < 1e-4, errs


def _symp_oracle64(S, shape, ce32, npml, faces, src, init, nsteps):
    """The FP64 oracle stepping the 4th-order scheme with the FP32 path's
    constants widened: coefficients, uniform ch, CPML tables, amplitudes."""
    w = lambda v: np.float64(np.float32(v))
    f = {k: init[k].astype(np.float64) for k in NAMES}
    ce = [c.astype(np.float64) for c in ce32]
    ch = w(S.COURANT / 24.0)
    tables = {}
    for coef in set(S.CL) | set(S.DL[:4]):
        t = [oracle.symp_stage_tables(p, coef, S.COURANT) if p else None for p in npml]
        tables[coef] = {k: [x[k].astype(np.float32).astype(np.float64) if x is not None else None for x in t]
                        for k in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}
    nx, ny, nz = shape
    ps = [(2 * npml[0], ny, nz), (nx, 2 * npml[1], nz), (nx, ny, 2 * npml[2])]
    psi_e = [np.zeros(ps[a]) if npml[a] else None for a in range(3) for _ in range(2)]
    psi_h = [np.zeros(ps[a]) if npml[a] else None for a in range(3) for _ in range(2)]
    pml = any(npml)

    def h_stage(cl):
        oracle.symp_h_scalar(w(cl), ch, *(f[k] for k in NAMES))
        if pml:
            oracle.symp_cpml_h(npml, faces, w(cl), ch, tables[cl], *(f[k] for k in NAMES), psi_h)

    for tn in range(1, nsteps + 1):
        for sn in range(4):
            h_stage(S.CL[sn])
            oracle.symp_e(w(S.DL[sn]), *(f[k] for k in NAMES), *ce)
            if pml:
                oracle.symp_cpml_e(npml, faces, w(S.DL[sn]), tables[S.DL[sn]], *(f[k] for k in NAMES), *ce, psi_e)
            for comp, (i, j, k), amp in src:
                f[comp][i, j, k] = f[comp][i, j, k] + w(amp(tn + sn / 5.0))
        h_stage(S.CL[4])
    return f, psi_e, psi_h


def test_symplectic_fp64_stage_bit_exact_vs_fp64_oracle():
    """The GPU FP64 4th-order stages (fdtd_symplectic_stage_f64, SympRun64)
    equal the FP64 C oracle bit for bit: CPML on all faces, a source, spheres,
    random initial state."""
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs, symplectic as S
    from fdtd_accelerate_gb300.fp64 import SympRun64
    F.build()
    shape, npml, nsteps = (26, 22, 30), 4, 4
    rng = np.random.default_rng(31)
    spheres = configs.random_spheres(rng, shape, 4, 2, 5, 1.0, 4.0)
    ce32 = [(c.numpy() * np.float32(S.COURANT / 24 / 0.5)).astype(np.float32)
            for c in configs.ce_from_spheres(shape, spheres)]
    amp = lambda t: np.sin(0.3 * t) * np.exp(-0.5 * ((t - 3.0) / 2.0) ** 2)
    src = [("ez", (13, 11, 15), amp)]
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    s32 = S.SymplecticSolver(shape, ce=ce32, npml=npml, sources=src, max_steps=nsteps + 2)
    r64 = SympRun64(s32)
    for q, k in enumerate(NAMES):
        r64.f[q].copy_(torch.from_numpy(init[k].astype(np.float64)))
    r64.step(nsteps)
    torch.cuda.synchronize()
    f, psi_e, psi_h = _symp_oracle64(S, shape, ce32, (npml,) * 3, 0x3F, src, init, nsteps)
    for q, k in enumerate(NAMES):
        np.testing.assert_array_equal(r64.f[q].cpu().numpy(), f[k], err_msg=k)
    for q in range(6):
        np.testing.assert_array_equal(r64.psi_e[q].cpu().numpy(), psi_e[q], err_msg="psi_e%d" % q)
        np.testing.assert_array_equal(r64.psi_h[q].cpu().numpy(), psi_h[q], err_msg="psi_h%d" % q)


def test_symp512_workload_fp32_vs_fp64_full_size():
    """The 4th-order workload at its own size (512^3, 10-cell CPML, 60 spheres
    eps_r U[1,4], centred Ez dipole), 1000 steps: the FP32 stage kernels against
    their FP64 twin on the GPU.  Per field family: max |a - b| / max |b| and
    the root-mean-square ratio."""
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    from fdtd_accelerate_gb300.fp64 import SympRun64, family_errors
    F.build()
    s32 = configs.symp512_solver(device="cuda", max_steps=1002)
    r64 = SympRun64(s32)
    s32.step(1000)
    r64.step(1000)
    torch.cuda.synchronize()
    errs = family_errors(s32.fields, r64.fields)
    print("symp512 workload, 1000 steps, FP32 vs FP64 (family-normalised max / rms):",
          ", ".join("%s %.2e / %.2e" % (k, errs[k]["max"], errs[k]["rms"]) for k in NAMES))
    assert max(e["max"] for e in errs.values()) < 3e-4, errs
    assert max(e["rms"] for e in errs.values()) < 1e-4, errs

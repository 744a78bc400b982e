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


def test_cpml_workload_fp32_vs_fp64():
    """The C2 workload scaled to 512x512x256 (12-cell CPML, spheres, dipoles),
    2000 steps: the fused FP32 path against the GPU FP64 step, same inputs.
    Reported per field family as max |a - b| / max |b|."""
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    from fdtd_accelerate_gb300.fp64 import YeeRun64
    F.build()
    shape, nsteps = (512, 512, 256), 2000
    work = configs.scaled(configs.cpml1024(steps=nsteps), shape)
    ce = configs.ce_from_spheres(shape, work.spheres, device="cuda")
    src = work.source_list(nsteps + 2)
    s32 = F.YeeSolver(shape, ce=ce, npml=12, sources=src)
    s32.step(nsteps)
    s64 = YeeRun64(shape, ce=ce, npml=12, sources=src)
    del ce
    s64.step(nsteps)
    torch.cuda.synchronize()
    s32.check_status()
    errs = {}
    for fam in (NAMES[:3], NAMES[3:]):
        scale = max(float(s64.fields[k].abs().max()) for k in fam)
        for k in fam:
            errs[k] = float((s32.fields[k].double() - s64.fields[k]).abs().max()) / scale
    print("cpml workload 512x512x256, %d steps, FP32 vs FP64 (family-normalised):" % nsteps,
          ", ".join("%s %.2e" % (k, errs[k]) for k in NAMES))
    # The FP32 path equals the reference's FP32 arithmetic bit for bit; this is
    # that arithmetic's distance to FP64 (measured 6e-5..1.1e-4 for E, 1e-5 for H).
    assert max(errs.values()) < 3e-4, errs

"""Parity cases run against the bounds-checked debug build.

Run as a child process with FDTD_GB300_CHECKED=1 (tests/test_gpu_checked.py):
the package then loads libfdtd_gb300_check.so, whose kernels compare every
wrapped global index with its array's extent.  Each case is a bit-exact
comparison between two paths of the library; at the end fdtd_debug_check must
report no index outside its array.  Prints one JSON line.
"""
import ctypes as C
import json
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


def _host(t):
    return t.detach().cpu().numpy()


def yee_cases(F, configs):
    """Fused step (TMA kernel, x/y CPML in kernel, z-band kernels) against the
    reference-shaped kernels: odd extents, ragged tiles, CPML on some faces."""
    for shape, npml, faces in [((37, 29, 45), 5, 0x3F), ((30, 26, 90), 6, 0x30), ((24, 40, 66), 4, 0x15)]:
        rng = np.random.default_rng(5)
        spheres = configs.random_spheres(rng, shape, 4, 2, 5, 1.0, 8.0)
        ce = [c.numpy() for c in configs.ce_from_spheres(shape, spheres)]
        t = np.arange(12, dtype=np.float64)
        src = [("ez", tuple(n // 2 for n in shape), F.gaussian_sine(t, 3.0, 2.0, 0.1)),
               ("ex", (npml + 1, 1, shape[2] - 2), F.gaussian_sine(t, 4.0, 2.0, 0.1))]
        init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
        a = F.YeeSolver(shape, ce=ce, npml=npml, faces=faces, sources=src)
        b = F.YeeSolver(shape, ce=ce, npml=npml, faces=faces, sources=src)
        a.set_fields(**init)
        b.set_fields(**init)
        a.step(6)
        b.step_unfused(6)
        torch.cuda.synchronize()
        a.check_status()
        for k in NAMES:
            np.testing.assert_array_equal(_host(a.fields[k]), _host(b.fields[k]), err_msg="yee %s %s" % (shape, k))
    return 3


def batch_case(F, configs):
    """Batched plan over ragged grids against single-grid plans."""
    grids = [((48, 32, 64), 8, 0x3F), ((37, 29, 45), 5, 0x15), ((20, 70, 36), 4, 0x3F)]
    solvers, refs = [], []
    for n, (shape, npml, faces) in enumerate(grids):
        rng = np.random.default_rng(40 + n)
        init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
        for lst in (solvers, refs):
            s = F.YeeSolver(shape, npml=npml, faces=faces)
            s.set_fields(**init)
            lst.append(s)
    batch = F.BatchSolver(solvers)
    batch.step(5)
    for s in refs:
        s.step(5)
    torch.cuda.synchronize()
    batch.check_status()
    for s, r in zip(solvers, refs):
        for k in NAMES:
            np.testing.assert_array_equal(_host(s.fields[k]), _host(r.fields[k]), err_msg="batch " + k)
    return 1


def symp_cases(S):
    """4th-order stage pairs (pair kernel inside, shell kernels) against the
    per-stage kernels, with merged H stages and sources on both parts."""
    n = 0
    for shape, npml, faces in [((40, 60, 132), 5, 0x3F), ((40, 36, 68), 5, 0x3F), ((30, 80, 68), 3, 0x0C)]:
        rng = np.random.default_rng(12)
        init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
        amp = lambda t: np.sin(0.3 * t) * np.exp(-0.5 * ((t - 4.0) / 2.0) ** 2)
        src = [("ez", tuple(v // 2 for v in shape), amp), ("ey", (shape[0] // 3, 2, 3), amp)]
        runs = []
        for fused in (True, False):
            s = S.SymplecticSolver(shape, npml=npml, faces=faces, sources=src, max_steps=5, fused=fused)
            s.set_fields(**init)
            s.step(3)
            runs.append(s)
        torch.cuda.synchronize()
        runs[0].check_status()
        for k in NAMES:
            np.testing.assert_array_equal(_host(runs[0].fields[k]), _host(runs[1].fields[k]),
                                          err_msg="symp %s %s" % (shape, k))
        n += 1
    return n


def main():
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import _native as N, configs
    from fdtd_accelerate_gb300 import symplectic as S
    assert N.CHECKED and N.LIB_PATH.endswith("libfdtd_gb300_check.so"), N.LIB_PATH
    cases = yee_cases(F, configs) + batch_case(F, configs) + symp_cases(S)
    torch.cuda.synchronize()
    word = C.c_uint64(0)
    N.call("fdtd_debug_check", C.byref(word))
    print(json.dumps({"cases": cases, "first_bad": int(word.value), "lib": os.path.basename(N.LIB_PATH)}), flush=True)


if __name__ == "__main__":
    main()

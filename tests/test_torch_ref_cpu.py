"""The FP64 autograd restatement (oracle/torch_ref.py) against the FP64 C
oracle, which the golden fixtures pin: same step, same CPML, same sources."""
import numpy as np
import pytest
import torch

import oracle
from oracle.torch_ref import TorchYee

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


@pytest.mark.parametrize("shape,npml,faces", [((14, 12, 16), (3, 3, 3), 0x3F), ((13, 15, 11), (2, 0, 3), 0x25),
                                              ((10, 10, 10), (0, 0, 0), 0x3F)])
def test_torch_step_matches_c_oracle(shape, npml, faces):
    rng = np.random.default_rng(5)
    tabs = [oracle.cpml_tables(p) if p else None for p in npml]
    ce = [rng.random(shape) * 0.5 for _ in range(3)]
    f = {k: rng.standard_normal(shape) for k in NAMES}
    for q, k in enumerate(("cex", "cey", "cez")):
        f[k] = ce[q]
    empty = {k: np.zeros(1) for k in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}
    tables = {k: [t[k] if t is not None else empty[k] for t in tabs] for k in empty}
    amp = np.sin(0.3 * np.arange(10))
    src = [("ez", (shape[0] // 2, shape[1] // 2, shape[2] // 2), amp)]
    sim = oracle.OracleSim({k: v.copy() for k, v in f.items()}, npml, faces, tables, src)
    ref = TorchYee(shape, npml, faces, [t if t is not None else None for t in tabs])
    E = [torch.from_numpy(f[k].copy()) for k in NAMES[:3]]
    H = [torch.from_numpy(f[k].copy()) for k in NAMES[3:]]
    _, _, pe, ph = ref.zero_state()
    cet = [torch.from_numpy(c) for c in ce]
    for t in range(1, 5):
        E, H, pe, ph = ref.step(E, H, pe, ph, cet, t, [(2, src[0][1], amp[t])])
    sim.step(4)
    for q, k in enumerate(NAMES):
        got = (E + H)[q].numpy()
        np.testing.assert_allclose(got, sim.f[k], rtol=0, atol=1e-12 * max(1.0, np.abs(sim.f[k]).max()),
                                   err_msg=k)
    for q in range(6):
        if sim.psi_e[q] is not None:
            np.testing.assert_allclose(pe[q].numpy(), sim.psi_e[q], rtol=0, atol=1e-12, err_msg="psi_e%d" % q)
            np.testing.assert_allclose(ph[q].numpy(), sim.psi_h[q], rtol=0, atol=1e-12, err_msg="psi_h%d" % q)


def test_torch_run_gradient_matches_fd():
    """Autograd through the FP64 restatement equals central differences."""
    shape, npml = (12, 11, 13), (3, 3, 3)
    ref = TorchYee(shape, npml, 0x3F, [oracle.cpml_tables(p) for p in npml])
    rng = np.random.default_rng(8)
    ce = torch.from_numpy(0.5 / (1.0 + 3.0 * rng.random((3,) + shape))).requires_grad_(True)
    amp = np.sin(0.4 * np.arange(40))
    src = [(2, (6, 5, 6), amp)]
    mons = [(2, (8, 7, 8)), (0, (4, 4, 9))]
    mon, _ = ref.run(list(ce), 30, src, mons, checkpoint_every=10)
    loss = (mon ** 2).sum()
    loss.backward()
    g = ce.grad
    for (q, i, j, k) in [(2, 7, 6, 7), (0, 5, 5, 8), (1, 6, 4, 6)]:
        h = 1e-6
        vals = []
        for sgn in (1, -1):
            c2 = ce.detach().clone()
            c2[q, i, j, k] += sgn * h
            m2, _ = ref.run(list(c2), 30, src, mons)
            vals.append(float((m2 ** 2).sum()))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - float(g[q, i, j, k])) <= 1e-6 * max(1.0, abs(fd)), (q, i, j, k, fd, float(g[q, i, j, k]))

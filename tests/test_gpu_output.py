"""Field output (kuFDTD Output: centred fields, Poynting vector, square / sum /
sqrt, spatial step, planes) on the GPU against the reference's own outputs and
the oracle, bit for bit."""
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


def test_output_matches_reference_golden(F, golden_dir):
    g = np.load(os.path.join(golden_dir, "output_kufdtd.npz"))
    fields = {k: torch.from_numpy(g["in_" + k]).cuda() for k in NAMES}
    for n in range(int(g["ncases"])):
        t = "c%d_" % n
        pts = g[t + "pts"]
        pt1 = tuple(None if v < 0 else int(v) for v in pts[0])
        pt2 = tuple(None if v < 0 else int(v) for v in pts[1])
        o = F.Output(str(g[t + "form"]), pt1, pt2, tuple(int(v) for v in pts[2]))
        o.set_space(fields)
        np.testing.assert_array_equal(o.get_data().cpu().numpy(), g[t + "out"], err_msg="case %d" % n)


@pytest.mark.parametrize("form", ["e", "h2", "ez", "hy2", "s", "s2", "sx", "sz2"])
def test_output_of_a_running_solver(F, form, tmp_path):
    """Padded solver fields (z pitch 36 for nz = 33) after a few steps of a
    CPML run with a source; a snapshot round-trips through .npy."""
    shape = (30, 28, 33)
    t = np.arange(20, dtype=np.float64)
    s = F.YeeSolver(shape, npml=5, sources=[("ez", (15, 14, 16), F.gaussian_sine(t, 3.0, 2.0, 0.2))])
    rng = np.random.default_rng(9)
    s.set_fields(**{k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES})
    s.step(6)
    torch.cuda.synchronize()
    host = {k: v.cpu().numpy() for k, v in s.fields.items()}
    for pt1, pt2, step in (((None,) * 3, (None,) * 3, (1, 1, 1)), ((3, 2, 5), (25, 20, 31), (2, 3, 4)),
                           ((4, None, None), (4, None, None), (1, 2, 1))):
        o = F.Output(form, pt1, pt2, step)
        o.set_space(s)
        got = o.get_data().cpu().numpy()
        np.testing.assert_array_equal(got, oracle.output_data(host, form, pt1, pt2, step), err_msg=str((pt1, step)))
    path = str(tmp_path / "snap.npy")
    o.save(path)
    np.testing.assert_array_equal(np.load(path), got)


def test_output_arguments(F):
    with pytest.raises(ValueError):
        F.Output("q", (1, 1, 1), (2, 2, 2))
    s = {k: torch.zeros((10, 10, 10), device="cuda") for k in NAMES}
    o = F.Output("e", (1, 1, 1), (9, 5, 5))      # p2 + 1 must stay inside the grid
    with pytest.raises(ValueError):
        o.set_space(s)

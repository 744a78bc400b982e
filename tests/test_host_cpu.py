"""Host-side set-up logic (no GPU): CPML tables, faces, workloads, sources."""
import numpy as np
import pytest
import torch

import oracle
from fdtd_accelerate_gb300 import configs
from fdtd_accelerate_gb300.cpml import cpml_tables, parse_faces, sigma_max_from_reflection
from fdtd_accelerate_gb300.sources import gaussian_sine


@pytest.mark.parametrize("npml", [1, 8, 10, 12])
def test_cpml_tables_match_oracle_restatement(npml):
    a = cpml_tables(npml)
    b = oracle.cpml_tables(npml)
    for k in a:
        np.testing.assert_allclose(a[k], b[k], rtol=1e-14, atol=1e-300, err_msg=k)


@pytest.mark.parametrize("npml", [1, 4, 10, 16])
def test_symplectic_stage_tables_match_oracle(npml):
    """The 4th-order stage CPML tables (sub-step coef*S per stage) agree with
    the oracle's restatement to FP64 rounding and are equal once rounded to
    the FP32 the kernels read, for every stage coefficient."""
    from fdtd_accelerate_gb300 import symplectic as S
    for coef in sorted(set(S.CL) | set(S.DL[:4])):
        a = S.stage_tables(npml, coef)
        b = oracle.symp_stage_tables(npml, coef)
        assert sorted(a) == sorted(b)
        for k in a:
            np.testing.assert_allclose(a[k], b[k], rtol=1e-14, atol=1e-15, err_msg="%s %r" % (k, coef))
            np.testing.assert_array_equal(np.asarray(a[k], np.float32), np.asarray(b[k], np.float32),
                                          err_msg="%s %r" % (k, coef))


def test_cpml_tables_reduce_to_non_kappa():
    """kappa_max = 1 gives km1 = 0 and a = sigma/(sigma+alpha)(b-1), the
    non-kappa coefficients of kuFDTD/v0.2.0/dim3/cpu/cpml.py:121-124."""
    t = cpml_tables(6, kappa_max=1.0)
    assert np.all(t["km1_e"] == 0) and np.all(t["km1_h"] == 0)
    P = 6
    smax = sigma_max_from_reflection(P)
    d = np.concatenate([P - np.arange(P) - 0.5, np.arange(P) + 0.5])
    sig = smax * (d / P) ** 4
    alp = 0.05 * (1 - d / P)
    b = np.exp(-(sig + alp) * 0.5)
    np.testing.assert_allclose(t["b_e"], b, rtol=1e-14)
    np.testing.assert_allclose(t["a_e"], sig / (sig + alp) * (b - 1), rtol=1e-12)


def test_parse_faces():
    assert parse_faces(("fb", "fb", "fb")) == 0x3F
    assert parse_faces(("+-", "", "-")) == 0x13
    assert parse_faces(("f", "b", "")) == 0x09
    with pytest.raises(ValueError):
        parse_faces(("x", "", ""))


def test_gaussian_sine():
    t = np.arange(400)
    a = gaussian_sine(t, 150, 30, 0.05)
    assert abs(a[150]) < 1e-12          # sin(2 pi 0.05 150) = sin(15 pi) = 0
    assert np.argmax(np.abs(a)) in range(140, 161)
    assert abs(a[0]) < 1e-5


def test_paint_spheres_and_ce():
    shape = (20, 22, 24)
    sph = [(10.0, 11.0, 12.0, 5, 4.0), (3.0, 3.0, 3.0, 2, 9.0)]
    eps = configs.paint_spheres(shape, sph, (0.5, 0.5, 0.0), dtype=torch.float64).numpy()
    assert eps[10, 11, 12] == 4.0 or eps[9, 10, 12] == 4.0
    assert eps.min() == 1.0 and eps.max() == 9.0
    ce = configs.ce_from_spheres(shape, sph)
    assert all(c.dtype == torch.float32 for c in ce)
    assert float(ce[0].max()) == 0.5
    np.testing.assert_allclose(float(ce[2].min()), 0.5 / 9.0, rtol=1e-6)


def test_workloads_seeded():
    a = configs.cpml1024(steps=10)
    b = configs.cpml1024(steps=10)
    assert a.spheres == b.spheres and a.dipoles == b.dipoles
    assert len(a.spheres) == 200 and len(a.dipoles) == 6
    for c, ijk, t0 in a.dipoles:
        assert c in ("ex", "ey", "ez") and 100 <= t0 <= 300
        for v, n in zip(ijk, a.shape):
            assert 14 <= v < n - 14
    s = configs.scaled(a, (64, 64, 32), steps=5)
    assert s.shape == (64, 64, 32) and len(s.spheres) == 200
    for c, ijk, t0 in s.dipoles:
        for v, n in zip(ijk, s.shape):
            assert 14 <= v <= n - 15

"""Pin the CPU oracle against outputs of the reference itself.

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py
from the reference's NumPy step (2nd_order-Yee/Numpy/fdtd3d.py), the KEMP
SSE/OpenMP core (KEMP/v0.7_pml/fdtd3d/cpu/src/core.c), the kuFDTD CPML C
routines (kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c), the kappa CPML
(kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c) and the 4th-order C
extension (4th_order-Symplectic/Python-C/dielectric.c).
"""
import os

import numpy as np
import pytest

import oracle

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


def _load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name + ".npz"))


def test_oracle_matches_numpy_reference_bit_exact(golden_dir):
    d = _load(golden_dir, "yee_numpy")
    for n in range(int(d["ncases"])):
        t = "c%d_" % n
        f = {k: d[t + "in_" + k].copy() for k in NAMES}
        ce = [d[t + "in_" + k] for k in ("cex", "cey", "cez")]
        nsteps, axes = d[t + "meta"]
        src = tuple(int(v) for v in d[t + "src"])
        for s in range(int(nsteps)):
            oracle.update_e(*(f[k] for k in NAMES), *ce)
            if axes:
                oracle.pbc_e(int(axes), f["ex"], f["ey"], f["ez"])
            f["ez"][src] = f["ez"][src] + d[t + "amps"][s]
            oracle.update_h(*(f[k] for k in NAMES))
            if axes:
                oracle.pbc_h(int(axes), f["hx"], f["hy"], f["hz"])
        for k in NAMES:
            np.testing.assert_array_equal(f[k], d[t + "out_" + k], err_msg="case %d %s" % (n, k))


def test_oracle_matches_kemp_core(golden_dir):
    """KEMP groups the curl as (a-b)-(c-d), NumPy as ((a-b)-c)+d: the two
    agree to a few ulp, so this check bounds the difference at 4 ulp of the
    largest term instead of bit equality."""
    d = _load(golden_dir, "kemp_core")
    for n in range(int(d["ncases"])):
        t = "c%d_" % n
        nz, pad, coeff, ufunc = (int(v) for v in d[t + "meta"])
        f = {k: d[t + "in_" + k].copy() for k in NAMES}
        if ufunc == 0:
            oracle.update_e(*(f[k] for k in NAMES), *(d[t + "in_" + k] for k in ("cex", "cey", "cez")))
            comps = NAMES[:3]
        else:
            ch = [d[t + "in_" + k] for k in ("chx", "chy", "chz")] if coeff else [None] * 3
            oracle.update_h(*(f[k] for k in NAMES), *ch)
            comps = NAMES[3:]
        for k in comps:
            ref = d[t + "out_" + k]
            tol = 4 * np.finfo(np.float32).eps * max(1.0, np.abs(ref).max())
            assert np.abs(f[k] - ref).max() <= tol, (n, k)


def test_oracle_cpml_matches_kufdtd_bit_exact(golden_dir):
    """With kappa = 1 (km1 = 0) the kappa-CPML restatement reduces exactly to
    the reference's non-kappa CPML."""
    d = _load(golden_dir, "cpml_kufdtd")
    for n in range(int(d["ncases"])):
        t = "c%d_" % n
        axis, which, backward, P = (int(v) for v in d[t + "meta"])
        E = [d[t + "in_" + k].copy() for k in NAMES[:3]]
        H = [d[t + "in_" + k].copy() for k in NAMES[3:]]
        CE = [d[t + "in_" + k] for k in ("cex", "cey", "cez")]
        npml = [0, 0, 0]
        npml[axis] = P
        faces = 1 << (2 * axis + backward)
        zero = np.zeros(2 * P)
        tables = {}
        for w in ("e", "h"):
            for name, val in (("b", d[t + "tb"]), ("a", d[t + "ta"]), ("km1", zero)):
                tables["%s_%s" % (name, w)] = [val if a == axis else None for a in range(3)]
        psi = [None] * 6
        psi[2 * axis] = d[t + "psi_in0"].copy()
        psi[2 * axis + 1] = d[t + "psi_in1"].copy()
        if which == 0:
            oracle.cpml_e(npml, faces, tables, *E, *H, *CE, psi)
            upd, comps = E, NAMES[:3]
        else:
            oracle.cpml_h(npml, faces, tables, *E, *H, psi)
            upd, comps = H, NAMES[3:]
        fm = d[t + "fmask"]
        pm = d[t + "pmask"]
        assert fm.any() and pm.any()
        for arr, k in zip(upd, comps):
            np.testing.assert_array_equal(arr[fm], d[t + "out_" + k][fm], err_msg="case %d %s" % (n, k))
        for r in range(2):
            np.testing.assert_array_equal(psi[2 * axis + r][pm], d[t + "psi_out%d" % r][pm],
                                          err_msg="case %d psi%d" % (n, r))


def test_oracle_kappa_cpml_matches_kufdtd(golden_dir):
    """The kappa CPML (kappa_max = 5) against the reference's own update_cpml_3d
    (kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c:238-265) on every axis,
    both faces, E and H.  psi = b psi + a d is single precision in both and
    must agree bit for bit.  The field correction differs in rounding: the
    reference evaluates cb ((1./kappa - 1) d + ds psi) in double (the literal
    1. promotes the expression) and rounds once when it adds the result to
    the float field, while the restatement (and every kernel) rounds each
    single-precision operation with km1 = 1/kappa - 1 rounded once from FP64.
    With the correction's terms of size c |km1 d| and c |psi| (their own
    roundings and the two km1 values differ by a few ulp of those terms), the
    bound per element is 4 ulp of the field plus 8 eps c_max (|km1|_max
    2 |base|_max + |psi|_max): a wrong sign, pairing or grouping of the kappa
    term would miss it by five orders of magnitude."""
    d = _load(golden_dir, "cpml_kappa_kufdtd")
    f32 = np.float32
    for n in range(int(d["ncases"])):
        t = "c%d_" % n
        axis, which, back, P = (int(v) for v in d[t + "meta"])
        npml = [0, 0, 0]
        npml[axis] = P
        faces = 1 << (2 * axis + back)
        tables = {}
        for w in ("e", "h"):
            for name, key in (("b", "tb"), ("a", "ta"), ("km1", "tkm1")):
                tables["%s_%s" % (name, w)] = [d[t + key] if a == axis else None for a in range(3)]
        psi = [None] * 6
        psi[2 * axis] = d[t + "psi_in0"].copy()
        psi[2 * axis + 1] = d[t + "psi_in1"].copy()
        E = [d[t + "in_" + k].copy() for k in NAMES[:3]]
        H = [d[t + "in_" + k].copy() for k in NAMES[3:]]
        if which == 0:
            oracle.cpml_e(npml, faces, tables, *E, *H, *(d[t + "in_" + k] for k in ("cex", "cey", "cez")), psi)
            upd, comps = E, NAMES[:3]
        else:
            oracle.cpml_h(npml, faces, tables, *E, *H, psi)
            upd, comps = H, NAMES[3:]
        base = E if which else H
        base_max = max(float(np.abs(x).max()) for x in base)
        psi_max = max(float(np.abs(psi[2 * axis + r]).max()) for r in range(2))
        km1_max = float(np.abs(d[t + "tkm1"]).max())
        c_max = 0.5 if which else max(float(np.abs(d[t + "in_" + k]).max()) for k in ("cex", "cey", "cez"))
        slack = 8 * np.finfo(f32).eps * c_max * (km1_max * 2 * base_max + psi_max)
        checked = 0
        for arr, k in zip(upd, comps):
            m = d[t + "fmask_" + k]
            if not m.any():
                continue
            ref_out, ref_in = d[t + "out_" + k][m], d[t + "in_" + k][m]
            corr = np.abs(ref_out.astype(np.float64) - ref_in)
            bound = 4 * np.spacing(np.maximum(np.abs(ref_out), np.abs(ref_in))) + slack
            err = np.abs(arr[m].astype(np.float64) - ref_out)
            assert (err <= bound).all(), "case %d %s: %g > bound" % (n, k, (err - bound).max())
            assert corr.max() > 1e3 * slack, "case %d %s: the kappa correction is not exercised" % (n, k)
            checked += 1
        assert checked == 2, n
        for r in range(2):
            pm = d[t + "pmask%d" % r]
            assert pm.any()
            np.testing.assert_array_equal(psi[2 * axis + r][pm], d[t + "psi_out%d" % r][pm],
                                          err_msg="case %d psi%d" % (n, r))


def test_oracle_symplectic_matches_reference_c_bit_exact(golden_dir):
    d = _load(golden_dir, "symp_c")
    for n in range(int(d["ncases"])):
        t = "c%d_" % n
        which = int(d[t + "meta"][0])
        f = [d[t + "in_" + k].copy() for k in NAMES]
        c = [d[t + "in_" + k] for k in ("c0", "c1", "c2")]
        coef = d[t + "coef"][()]
        if which == 0:
            oracle.symp_h(coef, *f, *c)
            comps = range(3, 6)
        else:
            oracle.symp_e(coef, *f, *c)
            comps = range(0, 3)
        for q in comps:
            np.testing.assert_array_equal(f[q][:-1, :-1, :-1], d[t + "out_" + NAMES[q]][:-1, :-1, :-1],
                                          err_msg="case %d %s" % (n, NAMES[q]))


def _drude_case(g, n):
    t = "c%d_" % n
    m = g[t + "meta"]
    E = [g[t + "in_" + k].copy() for k in ("ex", "ey", "ez")]
    CE = [g[t + "in_c" + k] for k in ("ex", "ey", "ez")]
    J = [g[t + "in_j" + a].copy() for a in "xyz"]
    CA = [g[t + "in_cja" + a] for a in "xyz"]
    CB = [g[t + "in_cjb" + a] for a in "xyz"]
    return t, tuple(int(v) for v in m[:3]), E, CE, J, CA, CB


def test_oracle_drude_matches_kufdtd_bit_exact(golden_dir):
    """Reference kuFDTD drude_ade.update_e (three calls, J carried over) on a
    sub-box and on the whole grid (tests/golden/drude_kufdtd.npz)."""
    g = np.load(os.path.join(golden_dir, "drude_kufdtd.npz"))
    for n in range(int(g["ncases"])):
        t, org, E, CE, J, CA, CB = _drude_case(g, n)
        for _ in range(3):
            oracle.drude_e(org, *E, *CE, J, CA, CB)
        for q, k in enumerate(("ex", "ey", "ez")):
            np.testing.assert_array_equal(E[q], g[t + "out_" + k], err_msg="case %d %s" % (n, k))
            np.testing.assert_array_equal(J[q], g[t + "out_j" + k[1]], err_msg="case %d J%s" % (n, k[1]))


def test_drude_coefficients_float32_arithmetic():
    """CJA, CJB as kuFDTD matter.py:198-208 evaluates them on float32 arrays."""
    rng = np.random.default_rng(4)
    w = rng.uniform(0.01, 0.5, (5, 6)).astype(np.float32)
    gam = rng.uniform(0.0, 0.3, (5, 6)).astype(np.float32)
    cja, cjb = oracle.drude_coefficients(w, gam, 0.5)
    assert cja.dtype == np.float32 and cjb.dtype == np.float32
    tmp = (2 + gam * np.float32(0.5)).astype(np.float32)
    np.testing.assert_array_equal(cja, ((2 - gam * np.float32(0.5)) / tmp).astype(np.float32))
    np.testing.assert_array_equal(cjb, (4 * (np.float32(0.5) * w) ** 2 / tmp).astype(np.float32))
    # no dispersion: J stays zero, E untouched
    cja0, cjb0 = oracle.drude_coefficients(np.zeros(3, np.float32), np.zeros(3, np.float32))
    np.testing.assert_array_equal(cja0, np.ones(3, np.float32))
    np.testing.assert_array_equal(cjb0, np.zeros(3, np.float32))


def test_oracle_fp64_matches_fp32_roughly():
    rng = np.random.default_rng(1)
    shape = (10, 11, 12)
    f32 = {k: rng.standard_normal(shape).astype(np.float32) for k in NAMES}
    f64 = {k: v.astype(np.float64) for k, v in f32.items()}
    ce = [np.full(shape, 0.5, np.float32) for _ in range(3)]
    for _ in range(20):
        oracle.update_e(*(f32[k] for k in NAMES), *ce)
        oracle.update_h(*(f32[k] for k in NAMES))
        oracle.update_e(*(f64[k] for k in NAMES), *(c.astype(np.float64) for c in ce))
        oracle.update_h(*(f64[k] for k in NAMES))
    for k in NAMES:
        err = np.abs(f32[k] - f64[k]).max() / np.abs(f64[k]).max()
        assert err < 1e-5


@pytest.mark.parametrize("npml", [4, 12])
def test_cpml_tables_shape_and_range(npml):
    t = oracle.cpml_tables(npml)
    for k in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h"):
        assert t[k].shape == (2 * npml,)
    assert np.all((t["b_e"] > 0) & (t["b_e"] <= 1))
    assert np.all(t["a_e"] <= 0)
    assert np.all((t["km1_e"] <= 0) & (t["km1_e"] > -1))
    # front slab is the mirror of the back slab
    np.testing.assert_allclose(t["b_e"][:npml][::-1], t["b_e"][npml:])
    np.testing.assert_allclose(t["b_h"][:npml][::-1], t["b_h"][npml:])


def test_oracle_tfsf_matches_kufdtd_bit_exact(golden_dir):
    """Reference kuFDTD Tfsf (executed in place by tests/golden/make_golden.py),
    12 updateE/updateH pairs from zero fields, every axis, all faces and a subset."""
    g = np.load(os.path.join(golden_dir, "tfsf_kufdtd.npz"))
    p1, p2 = [tuple(int(v) for v in r) for r in g["pt"]]
    shape = g["c0_out_ex"].shape
    for n in range(int(g["ncases"])):
        t = "c%d_" % n
        m = g[t + "meta"]
        axis, apply = int(m[0]), m[1:]
        faces = [bool(apply[a] & (1 if s == 0 else 2)) for a in range(3) for s in range(2)]
        ref = oracle.TfsfNormal(shape, p1, p2, faces, axis, 0.0, float(g["wdt"]))
        f = {k: np.zeros(shape, np.float32) for k in NAMES}
        for step in range(1, 13):
            ref.update_e(f, step)
            ref.update_h(f)
        for k in NAMES:
            np.testing.assert_array_equal(f[k], g[t + "out_" + k], err_msg="case %d %s" % (n, k))
        np.testing.assert_array_equal(ref.E, g[t + "e1d"])
        np.testing.assert_array_equal(ref.H, g[t + "h1d"])


def _output_case(g, n):
    t = "c%d_" % n
    pts = g[t + "pts"]
    pt1 = tuple(None if v < 0 else int(v) for v in pts[0])
    pt2 = tuple(None if v < 0 else int(v) for v in pts[1])
    return str(g[t + "form"]), pt1, pt2, tuple(int(v) for v in pts[2]), g[t + "out"]


def test_oracle_output_matches_kufdtd_bit_exact(golden_dir):
    """Reference kuFDTD Output.get_data() for all 24 dataforms on a stepped region
    and on a plane (tests/golden/output_kufdtd.npz)."""
    g = np.load(os.path.join(golden_dir, "output_kufdtd.npz"))
    fields = {k: g["in_" + k] for k in NAMES}
    for n in range(int(g["ncases"])):
        form, pt1, pt2, step, ref = _output_case(g, n)
        np.testing.assert_array_equal(oracle.output_data(fields, form, pt1, pt2, step), ref,
                                      err_msg="case %d %s" % (n, form))

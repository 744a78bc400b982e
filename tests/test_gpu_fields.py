"""KEMP-style object API on the GPU, following the reference's unit tests:
KEMP/v0.7_pml/fdtd3d/cpu/test/test_core.py (core vs naive after tmax updates),
test_incident_direct.py and test_get_set_fields.py (point/line/plane/volume
regions, scalar and array values)."""
import numpy as np
import pytest
import torch

import oracle
from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


@pytest.fixture(scope="module")
def K():
    import fdtd_accelerate_gb300 as F
    F.build()
    from fdtd_accelerate_gb300 import fields
    return fields


def two_points(rng, shape, ns):
    """Random regions as KEMP util/common_random.py:set_two_points draws them."""
    out = []
    def sorted_two(n):
        while True:
            a, b = np.sort(rng.integers(0, n, 2))
            if a != b:
                return int(a), int(b)
    for _ in range(2):
        if shape == "point":
            p = [int(rng.integers(0, n)) for n in ns]
            out.append((p, list(p)))
        elif shape == "line":
            for i, j, k in ((0, 1, 2), (2, 0, 1), (1, 2, 0)):
                p0, p1 = [0, 0, 0], [0, 0, 0]
                p0[i] = p1[i] = int(rng.integers(0, ns[i]))
                p0[j] = p1[j] = int(rng.integers(0, ns[j]))
                p0[k], p1[k] = sorted_two(ns[k])
                out.append((p0, p1))
        elif shape == "plane":
            for i, j, k in ((0, 1, 2), (2, 0, 1), (1, 2, 0)):
                p0, p1 = [0, 0, 0], [0, 0, 0]
                p0[i] = p1[i] = int(rng.integers(0, ns[i]))
                p0[j], p1[j] = sorted_two(ns[j])
                p0[k], p1[k] = sorted_two(ns[k])
                out.append((p0, p1))
        else:
            p0, p1 = zip(*(sorted_two(n) for n in ns))
            out.append((list(p0), list(p1)))
    return out


@pytest.mark.parametrize("ufunc", ["e", "h"])
@pytest.mark.parametrize("nz", [61, 62, 63, 64])
@pytest.mark.parametrize("coeff_use", ["", "e", "eh"])
def test_core_matches_oracle(K, ufunc, nz, coeff_use):
    """test_core.py:16-65: fields about to be updated start at zero, the others
    random; tmax updates; exact agreement with the oracle."""
    rng = np.random.default_rng(nz)
    nx, ny, tmax = 40, 50, 3
    ns = (nx, ny, nz)
    if ufunc == "e":
        ehs = [np.zeros(ns, np.float32) for _ in range(3)] + [rng.random(ns, dtype=np.float32) for _ in range(3)]
    else:
        ehs = [rng.random(ns, dtype=np.float32) for _ in range(3)] + [np.zeros(ns, np.float32) for _ in range(3)]
    ces = [rng.random(ns, dtype=np.float32) if "e" in coeff_use else np.full(ns, 0.5, np.float32) for _ in range(3)]
    chs = [rng.random(ns, dtype=np.float32) for _ in range(3)] if "h" in coeff_use else None
    fields = K.Fields(nx, ny, nz, coeff_use)
    K.Core(fields)
    fields.set_ehs(*ehs)
    fields.set_ces(*ces)
    if chs:
        fields.set_chs(*chs)
    ref = [a.copy() for a in ehs]
    for _ in range(tmax):
        if ufunc == "e":
            fields.update_e()
            oracle.update_e(*ref, *ces)
        else:
            fields.update_h()
            oracle.update_h(*ref, *(chs or (None,) * 3))
    fields.enqueue_barrier()
    for q, name in enumerate(NAMES):
        np.testing.assert_array_equal(fields.get(name).cpu().numpy(), ref[q], err_msg=name)
    # the z padding stays zero
    for name in NAMES:
        if fields.pad:
            assert float(fields._store[name][:, :, nz:].abs().max()) == 0.0


@pytest.mark.parametrize("shape", ["point", "line", "plane", "volume"])
def test_get_set_fields_roundtrip(K, shape):
    rng = np.random.default_rng(7)
    ns = (40, 50, 60)
    fields = K.Fields(*ns, "")
    ehs = [rng.random(ns, dtype=np.float32) for _ in range(6)]
    fields.set_ehs(*ehs)
    d = dict(zip(NAMES, ehs))
    for str_f in NAMES:
        for pt0, pt1 in two_points(rng, shape, ns):
            getf = K.GetFields(fields, str_f, pt0, pt1)
            getf.get_event().synchronize()
            sl = K.slices_two_points(pt0, pt1)
            np.testing.assert_array_equal(getf.get_fields(str_f).reshape(np.shape(d[str_f][sl])), d[str_f][sl])
    # multi-field get (boundary-exchange shapes of test_get_set_fields.py:226-234)
    nx, ny, nz = ns
    getf = K.GetFields(fields, ["ey", "ez"], (0, 0, 0), (0, ny - 2, nz - 2))
    getf.get_event().synchronize()
    np.testing.assert_array_equal(getf.get_fields("ez").reshape(ny - 1, nz - 1), ehs[2][0, :ny - 1, :nz - 1])
    # set: overwrite with an array, then add a scalar
    for str_f in ("ex", "hz"):
        for pt0, pt1 in two_points(rng, shape, ns):
            shp = K.shape_two_points(pt0, pt1)
            val = rng.random(shp, dtype=np.float32)
            K.SetFields(fields, str_f, pt0, pt1, is_array=True).set_fields(val)
            K.SetFields(fields, str_f, pt0, pt1, is_overwrite=False).set_fields(0.25)
            sl = K.slices_two_points(pt0, pt1)
            d[str_f][sl] = val.reshape(np.shape(d[str_f][sl]))
            d[str_f][sl] += np.float32(0.25)
            fields.enqueue_barrier()
            np.testing.assert_array_equal(fields.get(str_f).cpu().numpy(), d[str_f])


@pytest.mark.parametrize("is_array", [False, True])
def test_incident_direct(K, is_array):
    """test_incident_direct.py:16-41: one update_e/update_h puts
    f32(tfunc(1)) * value into the region of an all-zero field."""
    rng = np.random.default_rng(3)
    ns = (40, 50, 60)
    tfunc = lambda tstep: np.sin(0.03 * tstep)
    for str_f in NAMES:
        for shape in ("point", "line", "plane", "volume"):
            for pt0, pt1 in two_points(rng, shape, ns)[:2]:
                fields = K.Fields(*ns, "")
                sl = K.slices_two_points(pt0, pt1)
                if is_array:
                    value = rng.random(K.shape_two_points(pt0, pt1), dtype=np.float32)
                else:
                    value = float(rng.random())
                K.IncidentDirect(fields, str_f, pt0, pt1, tfunc, value)
                expect = np.zeros(ns, np.float32)
                v = np.float32(tfunc(1)) * (value if is_array else np.float32(value))
                expect[sl] = np.reshape(v, np.shape(expect[sl])) if is_array else v
                fields.update_e()
                fields.update_h()
                fields.enqueue_barrier()
                np.testing.assert_array_equal(fields.get(str_f).cpu().numpy(), expect)


def test_pml_and_priority_order(K):
    """Core, Pml, IncidentDirect appended in any order run as
    core < pml < incident (util/common.py:383-397) and equal the oracle."""
    ns = (30, 28, 36)
    fields = K.Fields(*ns, "e")
    src = K.IncidentDirect(fields, "ez", (15, 14, 18), (15, 14, 18), lambda t: np.sin(0.2 * t))
    pml = K.Pml(fields, ("+-", "+-", "+-"), npml=5)
    K.Core(fields)
    assert [type(i).__name__ for i in fields.instance_list] == ["Core", "Pml", "IncidentDirect"]
    rng = np.random.default_rng(9)
    ces = [(rng.random(ns, dtype=np.float32) * np.float32(0.5)) for _ in range(3)]
    fields.set_ces(*ces)
    tabs = [oracle.cpml_tables(5) for _ in range(3)]
    sim = oracle.OracleSim({**{k: np.zeros(ns, np.float32) for k in NAMES}, "cex": ces[0], "cey": ces[1],
                            "cez": ces[2]}, (5, 5, 5), 0x3F, {k: [t[k] for t in tabs] for k in tabs[0]},
                           [("ez", (15, 14, 18), np.float32(np.sin(0.2 * np.arange(20))))])
    for _ in range(12):
        fields.update_e()
        fields.update_h()
    sim.step(12)
    fields.enqueue_barrier()
    for name in NAMES:
        np.testing.assert_array_equal(fields.get(name).cpu().numpy(), sim.f[name], err_msg=name)
    assert src.tstep == 13 and pml.layer.active


def test_argument_errors(K):
    with pytest.raises(TypeError):
        K.Fields(40.0, 50, 60)
    with pytest.raises(ValueError):
        K.Fields(40, 50, 60, coeff_use="x")
    f = K.Fields(10, 12, 14, "")
    with pytest.raises(ValueError):
        f.get("ax")
    with pytest.raises(ValueError):
        K.GetFields(f, "ex", (0, 0, 0), (10, 0, 0))
    with pytest.raises(TypeError):
        K.IncidentDirect(f, "ex", (0, 0, 0), (1, 1, 1), 3.0)
    with pytest.raises(AttributeError):
        f.set_chs(*(np.zeros((10, 12, 14), np.float32),) * 3)

"""C ABI checks that need no GPU: the library loads, exports every entry
point declared in include/*.h, and rejects bad arguments before touching
CUDA (argument validation runs on the host)."""
import ctypes as C
import glob
import os
import re

import pytest

from tests.conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(fdtd_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from fdtd_accelerate_gb300 import _native, build
    build()
    return _native.lib()


def test_header_declares_entry_points():
    names = _declared()
    for n in ("fdtd_update_e_f32", "fdtd_update_h_f32", "fdtd_cpml_e_f32", "fdtd_cpml_h_f32",
              "fdtd_yee_plan_create", "fdtd_yee_plan_run", "fdtd_symplectic_h_f32"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(lib):
    from fdtd_accelerate_gb300 import _native as N
    for st in range(8):
        assert N.status_string(st)
    assert N.status_string(0) == "ok"


def test_debug_check_outside_the_checked_build(lib):
    """The product library is not the bounds-checked build: fdtd_debug_check
    reports that (no CUDA call) and writes 0."""
    import ctypes as C
    from fdtd_accelerate_gb300 import _native as N
    word = C.c_uint64(7)
    assert lib.fdtd_debug_check(C.byref(word)) == N.FDTD_ERR_UNSUPPORTED
    assert word.value == 0
    assert lib.fdtd_debug_check(None) == N.FDTD_ERR_ARG


def test_validation_before_cuda(lib):
    """Null pointers and inconsistent grids are rejected on the host."""
    from fdtd_accelerate_gb300 import _native as N
    g = N.Grid(4, 5, 6, 30, 6)
    null = [None] * 9
    assert lib.fdtd_update_e_f32(C.byref(g), *null, None) == N.FDTD_ERR_ARG
    bad = N.Grid(4, 5, 6, 29, 6)     # sx < ny*sy
    assert lib.fdtd_update_h_f32(C.byref(bad), *null, None) == N.FDTD_ERR_SHAPE
    bad = N.Grid(0, 5, 6, 30, 6)
    assert lib.fdtd_update_e_f32(C.byref(bad), *null, None) == N.FDTD_ERR_SHAPE
    assert lib.fdtd_update_pbc_e_f32(None, 1, None, None, None, None) == N.FDTD_ERR_ARG
    h = C.c_void_p()
    assert lib.fdtd_yee_plan_create(C.byref(h), C.byref(g), None, None, None, None, None, 0, None) == N.FDTD_ERR_ARG


def test_plan_rejects_unaligned_strides(lib):
    from fdtd_accelerate_gb300 import _native as N
    g = N.Grid(4, 5, 6, 30, 6)       # sy = 6 floats: rows not 16-byte aligned
    st = N.YeeState()
    for b in range(2):
        for q in range(6):
            st.f[b][q] = 0x1000 * (1 + q + 6 * b)
    for q in range(3):
        st.ce[q] = 0x100000 + 0x1000 * q
    h = C.c_void_p()
    status = C.c_int32(0)
    r = lib.fdtd_yee_plan_create(C.byref(h), C.byref(g), C.byref(st), None, None, None,
                                 C.byref(status), 0, None)
    assert r == N.FDTD_ERR_ALIGN


def test_error_mapping():
    from fdtd_accelerate_gb300 import _native as N
    with pytest.raises(ValueError):
        N.check(N.FDTD_ERR_SHAPE, "f")
    with pytest.raises(TimeoutError):
        N.check(N.FDTD_ERR_TIMEOUT, "f")
    with pytest.raises(NotImplementedError):
        N.check(N.FDTD_ERR_UNSUPPORTED, "f")
    with pytest.raises(RuntimeError):
        N.check(N.FDTD_ERR_CUDA, "f")


def test_drude_validation_before_cuda(lib):
    """A Drude box outside the grid or missing arrays is rejected on the host."""
    from fdtd_accelerate_gb300 import _native as N
    g = N.Grid(8, 9, 10, 90, 10)
    fake = [C.c_void_p(256 * (q + 1)) for q in range(6)]   # never dereferenced
    d = N.Drude(2, 3, 4, 4, 4, 4)
    assert lib.fdtd_drude_update_e_f32(C.byref(g), C.byref(d), *fake, None) == N.FDTD_ERR_ARG  # no J arrays
    for q in range(3):
        d.j[q] = d.cja[q] = d.cjb[q] = 512 * (q + 1)
    d.k0 = 7                                                # 7 + 4 > 10
    assert lib.fdtd_drude_update_e_f32(C.byref(g), C.byref(d), *fake, None) == N.FDTD_ERR_SHAPE
    d.k0, d.ni = 4, 0
    assert lib.fdtd_drude_update_e_f32(C.byref(g), C.byref(d), *fake, None) == N.FDTD_ERR_SHAPE
    assert lib.fdtd_drude_update_e_f32(C.byref(g), None, *fake, None) == N.FDTD_ERR_ARG


def test_tfsf_validation_before_cuda(lib):
    from fdtd_accelerate_gb300 import _native as N
    g = N.Grid(20, 20, 20, 400, 20)
    fake = [C.c_void_p(256 * (q + 1)) for q in range(3)]
    t = N.Tfsf()
    for a in range(3):
        t.p1[a], t.p2[a] = 5, 12
    t.faces, t.axis = 0x3F, 0
    assert lib.fdtd_tfsf_update_e_f32(C.byref(g), C.byref(t), 1, *fake, None) == N.FDTD_ERR_ARG  # no 1-D arrays
    t.e1d = t.h1d = t.abc = t.amp = 4096
    t.namp = 8
    t.p2[2] = 20                                            # p2 must stay below n
    assert lib.fdtd_tfsf_update_e_f32(C.byref(g), C.byref(t), 1, *fake, None) == N.FDTD_ERR_SHAPE
    t.p2[2] = 12
    assert lib.fdtd_tfsf_update_e_f32(C.byref(g), C.byref(t), 8, *fake, None) == N.FDTD_ERR_ARG  # past the table
    t.axis = 3
    assert lib.fdtd_tfsf_update_h_f32(C.byref(g), C.byref(t), *fake, None) == N.FDTD_ERR_ARG


def test_output_validation_before_cuda(lib):
    from fdtd_accelerate_gb300 import _native as N
    g = N.Grid(10, 10, 10, 100, 10)
    f = (C.c_void_p * 6)(*[256 * (q + 1) for q in range(6)])
    o = N.Output(0)
    for a in range(3):
        o.p1[a], o.p2[a], o.step[a] = 1, 8, 1
    out = C.c_void_p(4096)
    assert lib.fdtd_output_f32(C.byref(g), C.byref(o), f, out, 10, None) == N.FDTD_ERR_CAPACITY  # 512 cells
    o.p2[1] = 9                                                # 9 + 1 > n - 1
    assert lib.fdtd_output_f32(C.byref(g), C.byref(o), f, out, 1000, None) == N.FDTD_ERR_SHAPE
    o.p2[1], o.form = 8, 3 * 16                                # family 3 does not exist
    assert lib.fdtd_output_f32(C.byref(g), C.byref(o), f, out, 1000, None) == N.FDTD_ERR_ARG


def test_symplectic_stage_validation_before_cuda(lib):
    """fdtd_symplectic_stage_f32 rejects missing fields, a stage kind other
    than 0/1, an E stage without ce arrays, partial coefficient arrays, CPML
    without psi and slabs thicker than the axis allows, all on the host."""
    from fdtd_accelerate_gb300 import _native as N
    g = N.Grid(20, 20, 20, 400, 20)
    fake = C.c_void_p(16)  # never dereferenced: every case fails validation first
    f6 = (C.c_void_p * 6)(*([fake] * 6))
    c3 = (C.c_void_p * 3)(fake, fake, fake)
    part = (C.c_void_p * 3)(fake, None, fake)
    call = lib.fdtd_symplectic_stage_f32
    assert call(C.byref(g), None, 0, 0.5, 0.03, None, None, None, None) == N.FDTD_ERR_ARG
    assert call(C.byref(g), None, 2, 0.5, 0.03, f6, c3, None, None) == N.FDTD_ERR_ARG
    assert call(C.byref(g), None, 1, 0.5, 0.0, f6, None, None, None) == N.FDTD_ERR_ARG
    assert call(C.byref(g), None, 0, 0.5, 0.0, f6, part, None, None) == N.FDTD_ERR_ARG
    cp = N.Cpml()
    for a in range(3):
        cp.npml[a] = 4
        for key in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h"):
            getattr(cp, key)[a] = fake
    cp.faces = 0x3F
    assert call(C.byref(g), C.byref(cp), 1, 0.5, 0.0, f6, c3, None, None) == N.FDTD_ERR_ARG
    psi = N.Psi()
    for q in range(6):
        psi.e[q] = fake
        psi.h[q] = fake
    cp.npml[1] = 10  # 2P + 2 = 22 > ny = 20
    assert call(C.byref(g), C.byref(cp), 0, 0.5, 0.03, f6, None, C.byref(psi), None) == N.FDTD_ERR_SHAPE
    bad = N.Grid(20, 20, 20, 399, 20)
    assert call(C.byref(bad), None, 0, 0.5, 0.03, f6, None, None, None) == N.FDTD_ERR_SHAPE


def test_one_call_entry_points_validation_before_cuda(lib):
    """The one-call fused and batched entries reject a negative step count
    and missing descriptions on the host."""
    from fdtd_accelerate_gb300 import _native as N
    g = N.Grid(20, 20, 20, 400, 20)
    st = N.YeeState()
    assert lib.fdtd_yee_step_f32(C.byref(g), C.byref(st), None, None, None, 0, 1, -1, None, None) == N.FDTD_ERR_ARG
    assert lib.fdtd_yee_step_f32(None, C.byref(st), None, None, None, 0, 1, 2, None, None) == N.FDTD_ERR_ARG
    assert lib.fdtd_yee_step_f32(C.byref(g), C.byref(st), None, None, None, 0, 1, 2, None, None) == N.FDTD_ERR_ARG
    assert lib.fdtd_batched_run_f32(1, C.byref(g), C.byref(st), None, None, None, None, 0, 0, 1, -1, None,
                                    None) == N.FDTD_ERR_ARG


def _prototypes():
    """name -> parameter count of every function prototype in include/*.h"""
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(fdtd_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
            params = m.group(2).strip()
            out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def test_ctypes_signatures_match_header():
    """Every ctypes declaration in _native takes as many arguments as the C
    prototype it binds (a changed prototype cannot drift from its binding)."""
    from fdtd_accelerate_gb300 import _native as N
    protos = _prototypes()
    assert len(protos) >= 40
    for name, (_, args) in N._SIGS.items():
        assert name in protos, name
        assert len(args) == protos[name], (name, len(args), protos[name])

"""The allocation-free adjoint step (library-owned scratch) equals the
adjoint step with caller scratch over two calls in a row, and refuses a
CPML layer larger than its scratch."""
import ctypes as C

import numpy as np
import pytest
import torch

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def N():
    import fdtd_accelerate_gb300 as F
    F.build()
    from fdtd_accelerate_gb300 import _native
    return _native


def _case(N, shape, npml, seed, faces=0x3F):
    from fdtd_accelerate_gb300.cpml import CpmlLayer
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda")
    layer = CpmlLayer(shape, npml, faces)
    rnd = lambda s: torch.from_numpy(rng.standard_normal(s).astype(np.float32)).to(dev)
    nx, ny, nz = shape
    d = dict(layer=layer, lf=[rnd(shape) for _ in range(6)],
             lpe=[rnd(t.shape) if t is not None else None for t in layer.psi_e[0]],
             lph=[rnd(t.shape) if t is not None else None for t in layer.psi_h],
             hp=[[rnd(shape) for _ in range(3)] for _ in range(2)],
             pe=[[rnd(t.shape) if t is not None else None for t in layer.psi_e[0]] for _ in range(2)],
             ce=[(0.5 / (1 + 7 * torch.rand(shape, device=dev))).contiguous() for _ in range(3)],
             gce=[torch.zeros(shape, device=dev) for _ in range(3)],
             grid=N.Grid(nx, ny, nz, ny * nz, nz))
    return d


def _clone(d):
    c = dict(d)
    for k in ("lf", "lpe", "lph", "gce"):
        c[k] = [t.clone() if t is not None else None for t in d[k]]
    return c


def _run(N, d, fn, with_scratch):
    ptr = lambda t: t.data_ptr() if t is not None else None
    st = N.AdjointState()
    keep = []
    for q in range(6):
        st.lf[q] = ptr(d["lf"][q])
        st.lpsi_e[q], st.lpsi_h[q] = ptr(d["lpe"][q]), ptr(d["lph"][q])
        if with_scratch:
            we = torch.empty_like(d["lpe"][q]) if d["lpe"][q] is not None else None
            wh = torch.empty_like(d["lph"][q]) if d["lph"][q] is not None else None
            keep += [we, wh]
            st.w_e[q], st.w_h[q] = ptr(we), ptr(wh)
    for q in range(3):
        st.grad_ce[q] = ptr(d["gce"][q])
    cp = d["layer"].struct()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n in range(2):  # two calls in a row
        rc = getattr(N.lib(), fn)(C.byref(d["grid"]), C.byref(cp), C.byref(st),
                                  (C.c_void_p * 3)(*map(ptr, d["hp"][n])), (C.c_void_p * 6)(*map(ptr, d["pe"][n])),
                                  (C.c_void_p * 3)(*map(ptr, d["ce"])), None, None, stream)
        assert rc == 0, N.status_string(rc)
    torch.cuda.synchronize()
    return keep


@pytest.mark.parametrize("shape,npml", [((20, 18, 22), 4), ((33, 17, 40), 6), ((16, 16, 16), 0)])
def test_noalloc_matches_scratch_entry(N, shape, npml):
    d = _case(N, shape, npml, seed=len(shape) + npml)
    a, b = _clone(d), _clone(d)
    _run(N, a, "fdtd_adjoint_step_f32", True)
    _run(N, b, "fdtd_adjoint_step_noalloc_f32", False)
    for k in ("lf", "lpe", "lph", "gce"):
        for q, (x, y) in enumerate(zip(a[k], b[k])):
            if x is not None:
                assert torch.equal(x, y), "%s[%d]" % (k, q)


def test_noalloc_faces_off_after_other_layout(N):
    """Faces switched off (front faces only, 0x15) right after a call on another
    layout has left the shared scratch dirty: the back-face w entries are
    neither read nor written, so the result still equals the caller-scratch
    entry bit for bit."""
    warm = _case(N, (33, 17, 40), 6, seed=3)
    _run(N, _clone(warm), "fdtd_adjoint_step_noalloc_f32", False)
    d = _case(N, (24, 20, 28), 5, seed=11, faces=0x15)
    a, b = _clone(d), _clone(d)
    _run(N, a, "fdtd_adjoint_step_f32", True)
    _run(N, b, "fdtd_adjoint_step_noalloc_f32", False)
    for k in ("lf", "lpe", "lph", "gce"):
        for q, (x, y) in enumerate(zip(a[k], b[k])):
            if x is not None:
                assert torch.equal(x, y), "%s[%d]" % (k, q)


def test_noalloc_refuses_oversized_layer(N):
    nx, ny, nz = 300, 300, 100
    g = N.Grid(nx, ny, nz, ny * nz, nz)
    cp = N.Cpml()
    for a in range(3):
        cp.npml[a] = 20
    cp.faces = 0x3F
    st = N.AdjointState()
    rc = N.lib().fdtd_adjoint_step_noalloc_f32(C.byref(g), C.byref(cp), C.byref(st), None, None, None, None, None,
                                               None)
    assert rc == N.FDTD_ERR_CAPACITY

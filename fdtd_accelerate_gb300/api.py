"""Reference-shaped update functions on CUDA float32 tensors.

Drop-in for the positional array API of the reference:

    update_h(ex, ey, ez, hx, hy, hz)                    2nd_order-Yee/Numpy/fdtd3d.py:4-7
    update_e(ex, ey, ez, hx, hy, hz, cex, cey, cez)     2nd_order-Yee/Numpy/fdtd3d.py:10-13
    update_pbc_h(directions, hx, hy, hz)                2nd_order-Yee/Numpy/fdtd3d.py:20-29
    update_pbc_e(directions, ex, ey, ez)                2nd_order-Yee/Numpy/fdtd3d.py:31-40

Arrays are torch.float32 CUDA tensors of shape (nx, ny, nz) with unit z
stride (contiguous, or z-padded views such as ``Fields`` hands out).  They
are updated in place on the current CUDA stream; the functions return None,
like the reference's C extension (python-C/dielectric-sse-omp.c:57-60).
Bad arguments raise TypeError / ValueError as KEMP's checks do
(KEMP/v0.7_pml/fdtd3d/util/common.py:6-53); a missing native library
raises ImportError -- there is no CPU fallback.
"""
import ctypes as C

import torch

from . import _native as N

__all__ = ["update_e", "update_h", "update_pbc_e", "update_pbc_h", "grid_of", "stream_of",
           "check_field_tensors"]


def check_field_tensors(names, tensors):
    """Validate a group of field tensors: float32, CUDA, 3-D, one layout."""
    ref = None
    for name, t in zip(names, tensors):
        if not isinstance(t, torch.Tensor):
            raise TypeError("argument '%s' type must be a torch.Tensor : %s is given" % (name, type(t)))
        if t.dtype != torch.float32:
            raise TypeError("argument '%s' dtype must be torch.float32 : %s is given" % (name, t.dtype))
        if not t.is_cuda:
            raise ValueError("argument '%s' must be a CUDA tensor (no CPU fallback)" % name)
        if t.dim() != 3:
            raise ValueError("argument '%s' must be 3-D (nx, ny, nz) : shape %s" % (name, tuple(t.shape)))
        if t.stride(2) != 1 or t.stride(1) < t.shape[2] or t.stride(0) < t.shape[1] * t.stride(1):
            raise ValueError("argument '%s' must have unit z stride and non-overlapping rows : strides %s"
                             % (name, t.stride()))
        if ref is None:
            ref = (name, t)
        else:
            rn, rt = ref
            if t.shape != rt.shape or t.stride() != rt.stride():
                raise ValueError("argument '%s' shape/strides %s/%s differ from '%s' %s/%s"
                                 % (name, tuple(t.shape), t.stride(), rn, tuple(rt.shape), rt.stride()))
            if t.device != rt.device:
                raise ValueError("argument '%s' is on %s, '%s' on %s" % (name, t.device, rn, rt.device))
    return ref[1] if ref else None


def grid_of(t):
    nx, ny, nz = t.shape
    return N.Grid(nx, ny, nz, t.stride(0), t.stride(1))


def stream_of(t):
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def update_e(ex, ey, ez, hx, hy, hz, cex, cey, cez):
    names = ("ex", "ey", "ez", "hx", "hy", "hz", "cex", "cey", "cez")
    ts = (ex, ey, ez, hx, hy, hz, cex, cey, cez)
    ref = check_field_tensors(names, ts)
    g = grid_of(ref)
    with torch.cuda.device(ref.device):
        N.call("fdtd_update_e_f32", C.byref(g), *map(_ptr, ts), stream_of(ref))


def update_h(ex, ey, ez, hx, hy, hz, chx=None, chy=None, chz=None):
    names = ["ex", "ey", "ez", "hx", "hy", "hz"]
    ts = [ex, ey, ez, hx, hy, hz]
    chs = (chx, chy, chz)
    if any(c is not None for c in chs):
        if not all(c is not None for c in chs):
            raise ValueError("chx, chy, chz must be given together")
        names += ["chx", "chy", "chz"]
        ts += list(chs)
    ref = check_field_tensors(names, ts)
    g = grid_of(ref)
    with torch.cuda.device(ref.device):
        N.call("fdtd_update_h_f32", C.byref(g), *map(_ptr, (ex, ey, ez, hx, hy, hz, chx, chy, chz)),
               stream_of(ref))


def _axes(directions):
    if not isinstance(directions, str):
        raise TypeError("argument 'directions' type must be a str : %s is given" % type(directions))
    bad = set(directions) - set("xyz")
    if bad:
        raise ValueError("argument 'directions' may contain only 'x', 'y', 'z' : %r is given" % directions)
    return sum(b for a, b in (("x", 1), ("y", 2), ("z", 4)) if a in directions)


def update_pbc_e(directions, ex, ey, ez):
    axes = _axes(directions)
    ref = check_field_tensors(("ex", "ey", "ez"), (ex, ey, ez))
    g = grid_of(ref)
    with torch.cuda.device(ref.device):
        N.call("fdtd_update_pbc_e_f32", C.byref(g), axes, _ptr(ex), _ptr(ey), _ptr(ez), stream_of(ref))


def update_pbc_h(directions, hx, hy, hz):
    axes = _axes(directions)
    ref = check_field_tensors(("hx", "hy", "hz"), (hx, hy, hz))
    g = grid_of(ref)
    with torch.cuda.device(ref.device):
        N.call("fdtd_update_pbc_h_f32", C.byref(g), axes, _ptr(hx), _ptr(hy), _ptr(hz), stream_of(ref))

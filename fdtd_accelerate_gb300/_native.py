"""ctypes binding of libfdtd_gb300.so (the C ABI declared in include/fdtd_gb300.h).

The library is loaded from this package directory.  There is no CPU
fallback: if the library is missing or CUDA is unavailable, the calls raise.
With FDTD_GB300_CHECKED=1 in the environment the bounds-checked debug build
(libfdtd_gb300_check.so, buildlib.build(check=True)) is loaded instead.
"""
import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
CHECKED = os.environ.get("FDTD_GB300_CHECKED", "") == "1"
LIB_PATH = os.path.join(PKG, "libfdtd_gb300_check.so" if CHECKED else "libfdtd_gb300.so")

FDTD_OK = 0
FDTD_ERR_ARG = 1
FDTD_ERR_SHAPE = 2
FDTD_ERR_ALIGN = 3
FDTD_ERR_CUDA = 4
FDTD_ERR_TIMEOUT = 5
FDTD_ERR_UNSUPPORTED = 6
FDTD_ERR_CAPACITY = 7

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
F32 = C.c_float


class Grid(C.Structure):
    _fields_ = [("nx", I64), ("ny", I64), ("nz", I64), ("sx", I64), ("sy", I64)]


class Cpml(C.Structure):
    _fields_ = [("npml", I32 * 3), ("faces", I32),
                ("b_e", P * 3), ("a_e", P * 3), ("km1_e", P * 3),
                ("b_h", P * 3), ("a_h", P * 3), ("km1_h", P * 3)]


class Psi(C.Structure):
    _fields_ = [("e", P * 6), ("h", P * 6)]


class Sources(C.Structure):
    _fields_ = [("nsrc", I32), ("ijk", P), ("comp", P), ("amp", P), ("namp", I64)]


class Drude(C.Structure):
    _fields_ = [("i0", I64), ("j0", I64), ("k0", I64), ("ni", I64), ("nj", I64), ("nk", I64),
                ("j", P * 3), ("cja", P * 3), ("cjb", P * 3), ("j2", P * 3)]


class Tfsf(C.Structure):
    _fields_ = [("p1", I64 * 3), ("p2", I64 * 3), ("faces", I32), ("axis", I32), ("angle", C.c_double),
                ("e1d", P), ("h1d", P), ("abc", P), ("amp", P), ("namp", I64)]


class Output(C.Structure):
    _fields_ = [("form", I32), ("p1", I64 * 3), ("p2", I64 * 3), ("step", I64 * 3)]


class YeeState(C.Structure):
    _fields_ = [("f", (P * 6) * 2), ("psi_e", (P * 6) * 2), ("psi_h", P * 6), ("ce", P * 3), ("drude", P),
                ("tfsf", P)]


class SympState(C.Structure):
    _fields_ = [("f", (P * 6) * 2), ("psi_e", P * 6), ("psi_h", (P * 6) * 2), ("ce", P * 3)]


class Tile(C.Structure):
    _fields_ = [("tile_y", I32), ("x_chunk", I32), ("ctas_per_sm", I32), ("stages", I32), ("l2_promotion", I32)]


class Points(C.Structure):
    _fields_ = [("n", I32), ("ijk", P), ("comp", P)]


class AdjointState(C.Structure):
    _fields_ = [("lf", P * 6), ("lpsi_e", P * 6), ("lpsi_h", P * 6), ("w_e", P * 6), ("w_h", P * 6),
                ("grad_ce", P * 3)]


class FdtdError(RuntimeError):
    def __init__(self, status, fn, msg):
        super().__init__("%s failed: %s (status %d)" % (fn, msg, status))
        self.status = status


_SIGS = {
    "fdtd_status_string": (C.c_char_p, [C.c_int]),
    "fdtd_last_cuda_error": (C.c_int, []),
    "fdtd_update_e_f32": (C.c_int, [C.POINTER(Grid)] + [P] * 9 + [P]),
    "fdtd_update_h_f32": (C.c_int, [C.POINTER(Grid)] + [P] * 9 + [P]),
    "fdtd_update_pbc_e_f32": (C.c_int, [C.POINTER(Grid), I32, P, P, P, P]),
    "fdtd_update_pbc_h_f32": (C.c_int, [C.POINTER(Grid), I32, P, P, P, P]),
    "fdtd_cpml_e_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml)] + [P] * 9 + [C.POINTER(Psi), P]),
    "fdtd_cpml_h_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml)] + [P] * 9 + [C.POINTER(Psi), P]),
    "fdtd_add_sources_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Sources), I64, P, P, P, P]),
    "fdtd_drude_update_e_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Drude)] + [P] * 6 + [P]),
    "fdtd_tfsf_update_e_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Tfsf), I64, P, P, P, P]),
    "fdtd_output_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Output), P, P, I64, P]),
    "fdtd_tfsf_update_h_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Tfsf), P, P, P, P]),
    "fdtd_step_unfused_f32": (C.c_int, [C.POINTER(Grid), P, P, P, C.POINTER(Cpml), C.POINTER(Psi),
                                        C.POINTER(Sources), I64, P]),
    "fdtd_symplectic_h_f32": (C.c_int, [C.POINTER(Grid), F32] + [P] * 9 + [P]),
    "fdtd_symplectic_e_f32": (C.c_int, [C.POINTER(Grid), F32] + [P] * 9 + [P]),
    "fdtd_symplectic_h_scalar_f32": (C.c_int, [C.POINTER(Grid), F32, F32] + [P] * 6 + [P]),
    "fdtd_symplectic_cpml_e_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml), F32] + [P] * 9
                                   + [C.POINTER(Psi), P]),
    "fdtd_symplectic_cpml_h_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml), F32, F32] + [P] * 9
                                   + [C.POINTER(Psi), P]),
    "fdtd_symplectic_stage_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml), I32, F32, F32, C.POINTER(P * 6),
                                            C.POINTER(P * 3), C.POINTER(Psi), P]),
    "fdtd_yee_plan_create": (C.c_int, [C.POINTER(P), C.POINTER(Grid), C.POINTER(YeeState), C.POINTER(Cpml),
                                       C.POINTER(Sources), C.POINTER(Tile), P, I32, P]),
    "fdtd_yee_plan_run": (C.c_int, [P, I64, I64, P]),
    "fdtd_yee_plan_current": (C.c_int, [P]),
    "fdtd_yee_plan_set_current": (C.c_int, [P, I32]),
    "fdtd_yee_plan_test_timeout": (C.c_int, [P, I64, I32]),
    "fdtd_debug_check": (C.c_int, [C.POINTER(C.c_uint64)]),
    "fdtd_yee_plan_info": (C.c_int, [P, P, I32]),
    "fdtd_yee_plan_destroy": (C.c_int, [P]),
    "fdtd_yee_step_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(YeeState), C.POINTER(Cpml), C.POINTER(Sources), P,
                                    I32, I64, I64, C.POINTER(I32), P]),
    "fdtd_adjoint_step_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml), C.POINTER(AdjointState), P, P, P,
                                        C.POINTER(Points), P, P]),
    "fdtd_adjoint_step_noalloc_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml), C.POINTER(AdjointState), P, P,
                                                P, C.POINTER(Points), P, P]),
    "fdtd_adjoint_step_region_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml), C.POINTER(AdjointState), P, P,
                                               P, C.POINTER(Points), P, P, P]),
    "fdtd_gather_points_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Points), P, P, P]),
    "fdtd_step_unfused_f64": (C.c_int, [C.POINTER(Grid), P, P, C.POINTER(Cpml), P, P, C.POINTER(Sources), I64, P]),
    "fdtd_gather_points_f64": (C.c_int, [C.POINTER(Grid), C.POINTER(Points), P, P, P]),
    "fdtd_add_sources_f64": (C.c_int, [C.POINTER(Grid), C.POINTER(Sources), I64, P, P, P, P]),
    "fdtd_symplectic_stage_f64": (C.c_int, [C.POINTER(Grid), C.POINTER(Cpml), I32, C.c_double, C.c_double,
                                            C.POINTER(P * 6), C.POINTER(P * 3), C.POINTER(P * 6), P]),
    "fdtd_add_points_f32": (C.c_int, [C.POINTER(Grid), C.POINTER(Points), P, P, P]),
    "fdtd_symp_pair_plan_create": (C.c_int, [C.POINTER(P), C.POINTER(Grid), C.POINTER(SympState),
                                             C.POINTER(Sources), I32, I32, P, P, P]),
    "fdtd_symp_pair_run": (C.c_int, [P, C.POINTER(Cpml), C.POINTER(Cpml), C.POINTER(Cpml), F32, F32, I32, F32,
                                     F32, I64, P]),
    "fdtd_symp_pair_plan_current": (C.c_int, [P]),
    "fdtd_symp_pair_plan_set_current": (C.c_int, [P, I32]),
    "fdtd_symp_pair_plan_destroy": (C.c_int, [P]),
    "fdtd_batch_workspace_bytes": (C.c_size_t, [I32]),
    "fdtd_batch_plan_create": (C.c_int, [C.POINTER(P), I32, C.POINTER(Grid), C.POINTER(YeeState), C.POINTER(Cpml),
                                         C.POINTER(Sources), C.POINTER(Tile), P, P, C.c_size_t, I32, P]),
    "fdtd_batch_plan_run": (C.c_int, [P, I64, I64, P]),
    "fdtd_batch_plan_current": (C.c_int, [P]),
    "fdtd_batch_plan_set_current": (C.c_int, [P, I32]),
    "fdtd_batch_plan_info": (C.c_int, [P, P, I32]),
    "fdtd_batch_plan_destroy": (C.c_int, [P]),
    "fdtd_batched_run_f32": (C.c_int, [I32, C.POINTER(Grid), C.POINTER(YeeState), C.POINTER(Cpml),
                                       C.POINTER(Sources), P, P, C.c_size_t, I32, I64, I64, C.POINTER(I32), P]),
}

_lib = None


def lib():
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libfdtd_gb300.so not built: run "
                              "`python -c 'import __graft_entry__ as g; g.build()'` "
                              "or `python fdtd_accelerate_gb300/buildlib.py`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    L = lib()
    return [n for n in _SIGS if getattr(L, n, None) is not None]


def status_string(st):
    return lib().fdtd_status_string(st).decode()


def check(st, fn):
    if st == FDTD_OK:
        return
    msg = status_string(st)
    if st == FDTD_ERR_CUDA:
        msg += " (cudaError %d)" % lib().fdtd_last_cuda_error()
    if st in (FDTD_ERR_ARG, FDTD_ERR_SHAPE, FDTD_ERR_ALIGN, FDTD_ERR_CAPACITY):
        raise ValueError("%s failed: %s (status %d)" % (fn, msg, st))
    if st == FDTD_ERR_TIMEOUT:
        raise TimeoutError("%s failed: %s" % (fn, msg))
    if st == FDTD_ERR_UNSUPPORTED:
        raise NotImplementedError("%s failed: %s" % (fn, msg))
    raise FdtdError(st, fn, msg)


def call(name, *args):
    st = getattr(lib(), name)(*args)
    check(st, name)

"""ctypes binding of libflou_cuda (include/flou_cuda.h).

The shared library is built in-tree (flou.jl_gb300/lib/libflou_cuda.so).  There is no CPU
fallback: if the library is missing, every call raises FlouError.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# FLOU_CUDA_CHECKED=1 in the environment selects the build with device-side index checks
# (flou.jl_gb300/build.py --checked): slower, for tests; an out-of-range index is reported as
# FLOU_ERR_INDEX instead of being accessed.
CHECKED = os.environ.get("FLOU_CUDA_CHECKED", "") not in ("", "0")
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libflou_cuda_checked.so" if CHECKED else "libflou_cuda.so")

FLOU_OK = 0
FLOU_ERR_ARG = 1
FLOU_ERR_CUDA = 2
FLOU_ERR_NONPHYSICAL = 3
FLOU_ERR_TIMEOUT = 4
FLOU_ERR_OOM = 5
FLOU_ERR_UNSUPPORTED = 6
FLOU_ERR_STATE = 7
FLOU_ERR_INDEX = 8

EQ_LINEAR_ADVECTION, EQ_BURGERS, EQ_EULER = 0, 1, 2
OP_STRONG, OP_SPLIT, OP_HYBRID = 0, 1, 2
TP_STD_AVERAGE, TP_CHANDRASHEKAR, TP_KENNEDY_GRUBER = 0, 1, 2
NF_STD_AVERAGE, NF_LXF, NF_CHANDRASHEKAR, NF_HLL, NF_HLLC = 0, 1, 2, 3, 4
NF_SCALAR_DISSIPATION, NF_MATRIX_DISSIPATION = 5, 6
LIMITER_NONE, LIMITER_ZHANG_SHU = 0, 1
MONITOR_KINETIC_ENERGY, MONITOR_ENTROPY = 1, 2
BC_OUTFLOW, BC_INFLOW, BC_SLIP, BC_STATE_FIELD = 1, 2, 3, 4
PTR_HOST, PTR_DEVICE = 0, 1

STATUS_NAMES = {
    FLOU_ERR_ARG: "FLOU_ERR_ARG",
    FLOU_ERR_CUDA: "FLOU_ERR_CUDA",
    FLOU_ERR_NONPHYSICAL: "FLOU_ERR_NONPHYSICAL",
    FLOU_ERR_TIMEOUT: "FLOU_ERR_TIMEOUT",
    FLOU_ERR_OOM: "FLOU_ERR_OOM",
    FLOU_ERR_UNSUPPORTED: "FLOU_ERR_UNSUPPORTED",
    FLOU_ERR_STATE: "FLOU_ERR_STATE",
    FLOU_ERR_INDEX: "FLOU_ERR_INDEX",
}


class FlouError(RuntimeError):
    """A libflou_cuda call returned a non-zero status."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class DomainError(FlouError):
    """Non-physical state (rho <= 0, p <= 0, NaN), Flou's DomainError."""


class FlouConfig(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("equation", ctypes.c_int32),
        ("gamma", ctypes.c_double),
        ("advection", ctypes.c_double * 3),
        ("volume_op", ctypes.c_int32),
        ("twopoint_flux", ctypes.c_int32),
        ("numflux", ctypes.c_int32),
        ("numflux_avg", ctypes.c_int32),
        ("numflux_intensity", ctypes.c_double),
        ("nnodes", ctypes.c_int32),
    ]


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_I64 = ctypes.POINTER(ctypes.c_int64)

# Every symbol the header declares, with its argument types.
PROTOTYPES = {
    "flou_create": [ctypes.POINTER(FlouConfig), ctypes.POINTER(_P)],
    "flou_destroy": [_P],
    "flou_last_error": [_P],
    "flou_set_stream": [_P, _P],
    "flou_set_operators": [_P, _D, _D, _D, _D, _D, _D, _D, _D],
    "flou_set_mesh": [_P, ctypes.c_int32, ctypes.c_int32, _I32, _I32, _I32, _I32, _U8, _I32],
    "flou_set_bcs": [_P, ctypes.c_int32, _I32, _D],
    "flou_set_geometry": [_P, _D, _D, _D, _D],
    "flou_rhs": [_P, _P, _P, ctypes.c_double, ctypes.c_int32],
    "flou_step": [_P, _P, ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_int32],
    "flou_step_async": [_P, _P, ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_int32],
    "flou_wait": [_P],
    "flou_max_dt": [_P, _P, ctypes.c_double, _D, ctypes.c_int32],
    "flou_sizes": [_P, _I64, _I32, _I32, _I32],
    "flou_take_status": [_P, _I32, _I32],
    "flou_time_kernels": [_P, _P, ctypes.c_int32, _D, _D],
    "flou_rhs_noalloc": [_P, _P, _P, ctypes.c_double],
    "flou_fp64_peak": [_D],
    "flou_fp64_dmma_peak": [_D],
    "flou_check_refined_math": [ctypes.c_int64, _D, _D],
    "flou_set_dissipation": [_P, _P, ctypes.c_int32],
    "flou_check_mesh": [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _I32, _I32, _I32, _I32, _U8, _I32,
                        ctypes.c_char_p, ctypes.c_int32],
    "flou_check_geometry": [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _I32, _D, _D, _D, _D, _D,
                            ctypes.c_char_p, ctypes.c_int32],
    "flou_rhs_vjp": [_P, _P, _P, _P, _P],
    "flou_adjoint_solve": [_P, _P, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, _P, _P, _D, _P, _P, _I64],
    "flou_set_hybrid": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double],
    "flou_set_limiter": [_P, ctypes.c_int32, ctypes.c_double],
    "flou_set_bc_field": [_P, ctypes.POINTER(ctypes.c_double)],
    "flou_set_subgrid": [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    "flou_set_integrator": [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    "flou_step_cfl": [_P, _P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                      ctypes.c_int32, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)],
    "flou_limit": [_P, _P, ctypes.c_int32],
    "flou_monitor": [_P, _P, ctypes.c_int32, _D, ctypes.c_int32],
    "flou_set_monitors": [_P, ctypes.c_int32, ctypes.c_int32],
    "flou_take_monitors": [_P, _D, ctypes.c_int32, _I32],
    "flou_take_monitors_timed": [_P, _D, _D, ctypes.c_int32, _I32],
    "flou_adjoint_solve_batch": [ctypes.c_int32, ctypes.POINTER(_P), ctypes.POINTER(_P), _D, ctypes.c_int32,
                                 ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(_P), ctypes.POINTER(_P), _D,
                                 ctypes.POINTER(_P), ctypes.POINTER(_P), _I64, _I32],
    "flou_batch_create": [ctypes.c_int32, ctypes.POINTER(_P), ctypes.POINTER(_P)],
    "flou_batch_destroy": [_P],
    "flou_batch_last_error": [_P],
    "flou_batch_set_stream": [_P, _P],
    "flou_batch_set_states": [_P, ctypes.POINTER(_P), _D],
    "flou_batch_step": [_P, ctypes.c_int32],
    "flou_batch_autotune": [_P, _I32],
    "flou_batch_tiles": [_P, _I32],
    "flou_batch_set_tiles": [_P, _I32],
    "flou_batch_test_skip_faces": [_P, ctypes.c_int32],
}

_lib = None


def load():
    """Load libflou_cuda.so (raises FlouError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FlouError(FLOU_ERR_STATE, "libflou_cuda.so not built (%s); run build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_char_p if name.endswith("last_error") else ctypes.c_int32
    _lib = lib
    return lib


def check(status, ctx=None):
    if status == FLOU_OK:
        return
    msg = ""
    if ctx is not None:
        raw = load().flou_last_error(ctx)
        msg = raw.decode() if raw else ""
    cls = DomainError if status == FLOU_ERR_NONPHYSICAL else FlouError
    raise cls(status, msg)


def dptr(a):
    """ctypes double* of a C- or Fortran-contiguous float64 numpy array."""
    return a.ctypes.data_as(_D)

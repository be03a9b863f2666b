"""ctypes binding of libntk.so (the C ABI declared in include/ntk.h).

The library is loaded from this package directory.  There is no fallback:
if libntk.so is missing or cannot be loaded, every entry point raises.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libntk.so")

NTK_OK = 0
NTK_ERR_INVALID = 1
NTK_ERR_CUDA = 2
NTK_ERR_UNSUPPORTED = 3
NTK_ERR_RANGE = 4
NTK_ERR_TIMEOUT = 5
NTK_ERR_ALLOC = 6

NTK_STATUS_RANGE = 1

NTK_FP64 = 0
NTK_FP32 = 1
NTK_FP32_REFINE = 2

PRECISIONS = {"fp64": NTK_FP64, "fp32": NTK_FP32, "fp32_refine": NTK_FP32_REFINE}

NTK_TUNE_F64_X_VARIANT = 1
NTK_TUNE_F64_THREADS = 2
NTK_TUNE_REFINE_W = 3
NTK_TUNE_REFINE_SPW = 4
NTK_TUNE_REFINE_KERNEL = 5
NTK_TUNE_REFINE_PREFETCH = 6
NTK_TUNE_REFINE_TPS = 7
TUNE_KEYS = {"f64_x_variant": NTK_TUNE_F64_X_VARIANT, "f64_threads": NTK_TUNE_F64_THREADS,
             "refine_w": NTK_TUNE_REFINE_W, "refine_spw": NTK_TUNE_REFINE_SPW,
             "refine_kernel": NTK_TUNE_REFINE_KERNEL, "refine_prefetch": NTK_TUNE_REFINE_PREFETCH,
             "refine_tps": NTK_TUNE_REFINE_TPS}

# (name, restype, argtypes) of every exported entry point, in header order
_vp = ctypes.c_void_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_d = ctypes.c_double
SIGNATURES = [
    ("ntk_version", ctypes.c_char_p, []),
    ("ntk_last_error", _i, [ctypes.c_char_p, _i]),
    ("ntk_plan_create", _i, [ctypes.POINTER(_vp), _i, _ll, ctypes.POINTER(_d), _i, _i]),
    ("ntk_plan_set_tuning", _i, [_vp, _i, _i]),
    ("ntk_plan_get_tuning", _i, [_vp, _i, ctypes.POINTER(_i)]),
    ("ntk_plan_destroy", _i, [_vp]),
    ("ntk_plan_status", _i, [_vp, ctypes.POINTER(_i), _vp]),
    ("ntk_solve", _i, [_vp, _vp, _vp]),
    ("ntk_solve_strided", _i, [_vp, _vp, _vp, _ll, _ll, _ll, _ll, _ll, _vp]),
    ("ntk_compact_deriv", _i, [_vp, _vp, _vp, _i, _i, _i, _i, _d, _vp]),
    ("ntk_compact_grad", _i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _vp]),
    ("ntk_compact_rhs", _i, [_vp, _vp, _i, _i, _i, _d, _vp]),
    ("ntk_permute3d", _i, [_vp, _vp, _i, _i, _i, _ll, _ll, _ll, _vp]),
    ("ntk_adi_rhs", _i, [_vp, _vp, _i, _d, _d, _vp]),
    ("ntk_transpose2d", _i, [_vp, _vp, _i, _vp]),
    ("ntk_adi_create", _i, [ctypes.POINTER(_vp), _i, _d, _d, _i]),
    ("ntk_adi_destroy", _i, [_vp]),
    ("ntk_adi_status", _i, [_vp, ctypes.POINTER(_i), _vp]),
    ("ntk_adi_segments", _i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    ("ntk_adi_step", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("ntk_adi_run", _i, [_vp, _vp, _vp, _vp, _i, _i, _vp]),
    ("ntk_adi_var_create", _i, [ctypes.POINTER(_vp), _i, _d, _d, _vp, _vp, _i]),
    ("ntk_adi_var_destroy", _i, [_vp]),
    ("ntk_adi_var_step", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("ntk_adi_var_status", _i, [_vp, ctypes.POINTER(_i), _vp]),
    ("ntk_adi_step_static", _i, [_i, _d, _d, _vp, _vp, _vp, _vp]),
    ("ntk_batch_create", _i, [ctypes.POINTER(_vp), _ll, _vp, _vp, _vp, _vp, _vp, _i]),
    ("ntk_batch_destroy", _i, [_vp]),
    ("ntk_batch_status", _i, [_vp, ctypes.POINTER(_i), _vp]),
    ("ntk_batch_info", _i, [_vp, ctypes.POINTER(_ll), ctypes.POINTER(_ll), ctypes.POINTER(_ll)]),
    ("ntk_batch_windows", _i, [_vp, ctypes.POINTER(_ll), ctypes.POINTER(_ll)]),
    ("ntk_batch_solve", _i, [_vp, _vp, _vp]),
]

_lib = None
_lock = threading.Lock()


class NtkError(RuntimeError):
    """A libntk call returned a non-zero status."""

    def __init__(self, status, message):
        super().__init__("ntk status %d: %s" % (status, message))
        self.status = status


def load(path=None):
    """Load libntk.so (once).  Raises if it is missing: there is no CPU path."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError("libntk.so not found at %s; build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`" % p)
        lib = ctypes.CDLL(p)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(512)
    lib.ntk_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(status):
    if status != NTK_OK:
        msg = last_error()
        if status == NTK_ERR_INVALID:
            raise ValueError("ntk: " + msg)
        raise NtkError(status, msg)
    return status

"""ctypes binding of libtvgb.so (the C ABI declared in include/tvgb.h).

The library is the only compute path: if it is missing or fails to load,
every call raises; there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("TVGB_LIB") or os.path.join(HERE, "_build", "libtvgb.so")

TVGB_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "unsupported"}

LAYOUT_MAT3, LAYOUT_SYM6, LAYOUT_SYM6_PLANES = 9, 6, 60
EVEC_NONE, EVEC_CARTESIAN, EVEC_SPHERICAL = 0, 1, 2
EIG_PARITY, EIG_PRECISE = 0, 1

_P = ctypes.c_void_p
_U = ctypes.c_uint
_I = ctypes.c_int
_F = ctypes.c_float
_SZ = ctypes.c_size_t


class Vote3Params(ctypes.Structure):
    """tvgb_vote3_params (include/tvgb.h)."""
    _fields_ = [("sigma1", ctypes.c_float), ("sigma2", ctypes.c_float), ("w", ctypes.c_uint),
                ("power", ctypes.c_uint), ("samples", ctypes.c_uint), ("stick", ctypes.c_int),
                ("plate", ctypes.c_int), ("ball", ctypes.c_int), ("is_atv", ctypes.c_int),
                ("parity", ctypes.c_int)]


SIGNATURES = {
    "tvgb_last_error": (ctypes.c_char_p, []),
    "tvgb_version": (_I, []),
    "tvgb_launch_count": (ctypes.c_ulonglong, []),
    "tvgb_memory_stats": (_I, [_P, _P, ctypes.c_int]),
    "tvgb_surrogate_param_count": (_I, []),
    "tvgb_surrogate_samples": (_I, [_SZ, ctypes.c_ulonglong, _P, _P, _P]),
    "tvgb_surrogate_grad": (_I, [_P, _P, _P, _I, _P, _P, _P]),
    "tvgb_surrogate_train": (_I, [_P, _P, _P, _SZ, _I, _I, _F, _P, _P]),
    "tvgb_surrogate_eval": (_I, [_P, _P, _SZ, _P, _P]),
    "tvgb_surrogate_eval_tc": (_I, [_P, _P, _SZ, _P, _I, _P]),
    "tvgb_surrogate_eval_tc_limit": (_I, [_P, _P, _SZ, _P, _I, ctypes.c_longlong, _P]),
    "tvgb_vote3_surrogate": (_I, [_P, _I, _U, _U, _U, ctypes.POINTER(Vote3Params), _P, _I, _F, _P, _I, _P, _P, _I,
                                  _P, _P]),
    "tvgb_stick_saliency2": (_I, [_P, _SZ, _P, _P]),
    "tvgb_otsu_threshold": (_I, [_P, _SZ, _P, _P]),
    "tvgb_saliency_threshold2": (_I, [_P, ctypes.c_uint, ctypes.c_uint, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_int, _P, _P, _P]),
    "tvgb_simf2": (_I, [_P, _P, _SZ, _P, _P]),
    "tvgb_tensorvote_sweep": (_I, [_P, _P, ctypes.c_uint, ctypes.c_uint, _P, ctypes.c_int, ctypes.c_uint, ctypes.c_int,
                                   _P, _P, _P]),
    "tvgb_evals3_symmetric": (_I, [_P, _SZ, _P, _P]),
    "tvgb_evecs3spherical_symmetric": (_I, [_P, _P, _SZ, _P, _P]),
    "tvgb_evals2_symmetric": (_I, [_P, _SZ, _P, _P]),
    "tvgb_evecs2polar_symmetric": (_I, [_P, _P, _SZ, _P, _P]),
    "tvgb_eig3": (_I, [_P, _I, _SZ, _P, _P, _I, _I, ctypes.POINTER(ctypes.c_size_t), _P]),
    "tvgb_gaussian_filter3d": (_I, [_P, _U, _U, _U, _F, _F, _F, _P, _P, _P]),
    "tvgb_gaussian_convolve2": (_I, [_P, _U, _U, _F, _F, _P, _P, _P]),
    "tvgb_structure_tensor3": (_I, [_P, _U, _U, _U, _F, _I, _P, _I, _P, _P]),
    "tvgb_structure_tensor2": (_I, [_P, _U, _U, _F, _I, _P, _P, _P]),
    "tvgb_tensorvote3": (_I, [_P, _P, _U, _U, _U, _F, _F, _U, _U, _I, _I, _I, _U, _I, _P]),
    "tvgb_tensorvote": (_I, [_P, _P, _F, _F, _I, _U, _U, _U, _I, _I, _U, _I, _P]),
    "tvgb_tensorvote_prebuilt": (_I, [_P, _P, _P, _I, _F, _F, _I, _U, _U, _U, _I, _I, _U, _P]),
    "tvgb_build_neighbors2d": (_I, [_I, _F, _F, _U, _U, _I, _I, _P, ctypes.POINTER(ctypes.c_int)]),
    "tvgb_build_neighbors3d": (_I, [_I, _F, _F, _P, ctypes.POINTER(ctypes.c_int)]),
    "tvgb_vote3": (_I, [_P, _I, _U, _U, _U, ctypes.POINTER(Vote3Params), _P, _I, _P, _P, _I, _P]),
    "tvgb_vote3_noalloc": (_I, [_P, _I, _U, _U, _U, ctypes.POINTER(Vote3Params), _P, _I, _P, _P, _I, _P]),
    "tvgb_pipeline3": (_I, [_P, _U, _U, _U, _F, _I, ctypes.POINTER(Vote3Params), _P, _I, _P, _P, _I, _P, _P]),
    "tvgb_sticknorm3": (ctypes.c_double, [_F, _F, _U]),
    "tvgb_profile_enable": (_I, [_I]),
    "tvgb_profile_read": (_I, [ctypes.c_char_p, _SZ]),
    "tvgb_fp32_peak": (_I, [_P, _P, _P]),
    "tvgb_release_cached_memory": (_I, []),
    "tvgb_pipe_rates": (_I, [_P, _P]),
}

_lib = None


class TvgbError(RuntimeError):
    """A libtvgb call returned a non-zero status."""

    def __init__(self, fn, status, message):
        super().__init__(f"{fn}: {ERRORS.get(status, status)}: {message}")
        self.status = status


def lib():
    """The loaded library; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libtvgb.so not found at {LIB_PATH}: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def call(name, *args):
    """Call a status-returning entry point; raise TvgbError on failure."""
    st = getattr(lib(), name)(*args)
    if st != TVGB_OK:
        msg = lib().tvgb_last_error()
        raise TvgbError(name, st, msg.decode() if msg else "")
    return st

"""ctypes binding of libgpp_gb300.so (the C ABI in include/gpp_gb300.h).

Loading fails loudly when the library has not been built: there is no
fallback implementation behind this module.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

GPP_OK = 0
GPP_ERR_INVALID_ARGUMENT = 1
GPP_ERR_CUDA = 2
GPP_ERR_OUT_OF_MEMORY = 3
GPP_ERR_UNSUPPORTED = 4
GPP_ERR_BAD_INDEX = 5
GPP_ERR_NOT_READY = 6
GPP_ERR_DEVICE_TIMEOUT = 7

PRECISION = {"fp64": 0, "mixed": 1}
SEMANTICS = {"complex_seq": 0, "kerseq": 1}

_vp = C.c_void_p
_i = C.c_int
_d = C.c_double


class GppProblem(C.Structure):
    _fields_ = [("number_bands", _i), ("nvband", _i), ("ncouls", _i), ("ngpown", _i), ("nw", _i),
                ("aqsmtemp", _vp), ("aqsntemp", _vp), ("I_eps_array", _vp), ("wtilde_array", _vp),
                ("vcoul", _vp), ("inv_igp_index", _vp), ("indinv", _vp), ("wx_array", _vp),
                ("wx_stride", _i), ("occ", _d), ("semantics", _i), ("precision", _i)]


class GppOutputs(C.Structure):
    _fields_ = [("achtemp", _vp), ("asxtemp", _vp), ("acht_n1_loc", _vp), ("achstemp", _vp)]


# name -> (restype, argtypes)
_SIGS = {
    "gpp_kernel_gpu": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp]),
    "gpp_till_nvband": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d]),
    "gpp_noflag_occ_solver": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gpp_reduce_achstemp": (_i, [_i, _vp, _i, _vp, _vp, _vp, _vp, _i, _vp]),
    "gpp_reduce_achstemp_split": (_i, [_i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "gpp_set_stream": (_i, [_vp]),
    "gpp_get_stream": (_vp, []),
    "gpp_sigma": (_i, [C.POINTER(GppProblem), C.POINTER(GppOutputs), _vp]),
    "gpp_wait": (_i, [_vp, _i]),
    "gpp_context_create": (_i, [C.POINTER(_vp)]),
    "gpp_context_destroy": (_i, [_vp]),
    "gpp_sigma_host": (_i, [_vp, C.POINTER(GppProblem), C.POINTER(GppOutputs)]),
    "gpp_sigma_batched": (_i, [C.POINTER(GppProblem), C.POINTER(GppOutputs), _i, _vp]),
    "gpp_batch_create": (_i, [C.POINTER(_vp), C.POINTER(GppProblem), C.POINTER(GppOutputs), _i]),
    "gpp_batch_run": (_i, [_vp, _vp]),
    "gpp_batch_destroy": (_i, [_vp]),
    "gpp_sigma_static_scratch": (_i, [C.POINTER(GppProblem), C.POINTER(GppOutputs), _vp]),
    "gpp_autotune": (_i, [C.POINTER(GppProblem), _i, _vp, C.POINTER(_i)]),
    "gpp_set_variant": (_i, [_i, _i]),
    "gpp_tuned_variant": (_i, [_i, C.POINTER(_i)]),
    "gpp_variant_count": (_i, []),
    "gpp_variant_name": (C.c_char_p, [_i]),
    "gpp_last_error_message": (C.c_char_p, []),
    "gpp_launch_count": (C.c_ulonglong, []),
    "gpp_reset_launch_count": (None, []),
    "gpp_enable_kernel_timing": (_i, [_i]),
    "gpp_last_kernel_ms": (_i, [C.POINTER(C.c_float)]),
    "gpp_probe_fma_peaks": (_i, [C.POINTER(_d), C.POINTER(_d)]),
    "gpp_context_last_timing": (_i, [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                     C.POINTER(C.c_float)]),
    "gpp_context_last_trace": (_i, [_vp, C.POINTER(C.c_float), _i, C.POINTER(_i)]),
    "gpp_selftest_wait_timeout": (_i, [_i, _vp]),
    "gpp_set_dropin_precision": (_i, [_i]),
    "gpp_get_dropin_precision": (_i, []),
    "gpp_set_gemm_path": (_i, [_i]),
}

_lib = None


def library_path() -> str:
    return _build.LIB


def load() -> C.CDLL:
    """Load libgpp_gb300.so (RuntimeError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() "
                           "(the GB300 kernels have no fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GppError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = load().gpp_last_error_message().decode(errors="replace")
        super().__init__(f"{where} failed with status {status}: {msg}")
        self.status = status


def check(status: int, where: str) -> None:
    if status != GPP_OK:
        raise GppError(status, where)

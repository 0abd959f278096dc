"""The C-ABI library without a GPU: it builds, loads, exports every symbol
include/gpp_gb300.h declares (plus the reference's C++ entry points) and
rejects bad arguments before touching the device."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import REPO
from gppsigma import build, capi

HEADER = os.path.join(REPO, "include", "gpp_gb300.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gpp_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_reference_cpp_entry_points_are_exported(lib):
    out = subprocess.run(["nm", "-DC", "--defined-only", capi.library_path()],
                         capture_output=True, text=True, check=True).stdout
    for sig in ("d_till_nvband(int, int, int, int*, double*, GPPComplex*, GPPComplex*, "
                "GPPComplex*, GPPComplex*, GPPComplex*, double*, GPPComplex*, double*, double*, double)",
                "d_noFlagOCCSolver(int, int, int, int, int*, double*, GPPComplex*, GPPComplex*, "
                "GPPComplex*, GPPComplex*, double*, double*, double*, GPPComplex*)",
                "gppKernelGPU(GPPComplex*, GPPComplex*, GPPComplex*, GPPComplex*, int, int, int, "
                "double*, double*, double*, double*, int, int, int*, int*)",
                "d_reduce_achstemp(int, int*, int, GPPComplex*, GPPComplex*, GPPComplex*, double*, "
                "double*, int, double*)"):
        assert sig in out, sig


def test_invalid_arguments_are_reported_without_a_device(lib):
    assert lib.gpp_sigma(None, None, None) == capi.GPP_ERR_INVALID_ARGUMENT
    assert b"NULL" in lib.gpp_last_error_message()
    p = capi.GppProblem()
    p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nw = 4, 5, 10, 2, 3
    o = capi.GppOutputs()
    assert lib.gpp_sigma(C.byref(p), C.byref(o), None) == capi.GPP_ERR_INVALID_ARGUMENT
    assert b"nvband" in lib.gpp_last_error_message()
    p.nvband, p.ncouls = 1, 0
    assert lib.gpp_sigma(C.byref(p), C.byref(o), None) == capi.GPP_ERR_INVALID_ARGUMENT
    p.ncouls, p.wx_stride = 10, 2
    assert lib.gpp_sigma(C.byref(p), C.byref(o), None) == capi.GPP_ERR_INVALID_ARGUMENT
    p.wx_stride, p.precision = 0, 7
    assert lib.gpp_sigma(C.byref(p), C.byref(o), None) == capi.GPP_ERR_INVALID_ARGUMENT
    # Reference-signature entry points validate too (NULL arrays, nend <= nstart).
    assert lib.gpp_kernel_gpu(None, None, None, None, 10, 2, 4, None, None, None, None, 0, 3,
                              None, None) == capi.GPP_ERR_INVALID_ARGUMENT
    assert lib.gpp_till_nvband(2, 2, 10, None, None, None, None, None, None, None, None, None,
                               None, None, 1.0) == capi.GPP_ERR_INVALID_ARGUMENT
    assert lib.gpp_noflag_occ_solver(4, 2, 2, 10, None, None, None, None, None, None, None,
                                     None, None, None) == capi.GPP_ERR_INVALID_ARGUMENT
    assert lib.gpp_context_create(None) == capi.GPP_ERR_INVALID_ARGUMENT
    assert lib.gpp_sigma_batched(None, None, -1, None) == capi.GPP_ERR_INVALID_ARGUMENT


def test_path_and_precision_setters_validate(lib):
    assert lib.gpp_set_gemm_path(3) == capi.GPP_ERR_INVALID_ARGUMENT
    assert lib.gpp_set_gemm_path(-2) == capi.GPP_ERR_INVALID_ARGUMENT
    for mode in (2, 1, 0, -1):
        assert lib.gpp_set_gemm_path(mode) == capi.GPP_OK
    assert lib.gpp_set_dropin_precision(3) == capi.GPP_ERR_INVALID_ARGUMENT
    assert lib.gpp_set_dropin_precision(-1) == capi.GPP_OK


def test_stream_setter_round_trip(lib):
    assert lib.gpp_set_stream(C.c_void_p(0x1234)) == capi.GPP_OK
    assert lib.gpp_get_stream() == 0x1234
    assert lib.gpp_set_stream(None) == capi.GPP_OK
    assert not lib.gpp_get_stream()


def test_launch_counter_resets(lib):
    lib.gpp_reset_launch_count()
    assert lib.gpp_launch_count() == 0

"""gpp_sigma_static_scratch: the allocation-free FP64 entry point.

Some callers cannot allocate device memory -- applications that have given
the GPU's memory to their own arena or to another runtime, or that cannot
take cudaMalloc's device-wide synchronisation mid-step.  This entry point
keeps its scratch in a fixed array inside the library.  Checked here through
the C ABI against gpp_sigma on the same inputs, on two calls in a row (the
second call starts from the first call's leftover scratch contents), plus the
size limit.  The file sorts last so that a failure here cannot hide others."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from gppsigma import build, capi, workload as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FP64_TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()
    capi.load()


def _outputs(nw):
    a = torch.zeros(nw, dtype=torch.complex128, device="cuda")
    b = torch.zeros(nw, dtype=torch.complex128, device="cuda")
    o = capi.GppOutputs()
    o.achtemp, o.asxtemp = a.data_ptr(), b.data_ptr()
    return o, a, b


def _inputs(shape, seed, band_independent=False, indinv=False):
    import dataclasses
    inp = W.make_inputs(shape, seed)
    if band_independent:
        inp.wx_array = inp.wx_array[:1].copy()
    if indinv:
        perm = np.random.default_rng(seed).permutation(shape.ncouls).astype(np.int32)
        inp = dataclasses.replace(inp, indinv=perm)
    return inp


# (shape, seed, band-independent wx, non-identity indinv, bit-identical to gpp_sigma)
CASES = [
    (W.Shape(40, 3, 3000, 57, 3), 1, False, False, True),
    (W.Shape(17, 2, 1500, 21, 5, near_pole=0.02), 2, False, False, True),
    # indinv remaps the clamped igp (GPPComplex.h:304): same kernels, same bits.
    (W.Shape(12, 2, 800, 21, 3, near_pole=0.02, igp_overflow=3), 3, False, True, True),
    # Band-independent wx with >= 32 unoccupied bands: gpp_sigma sums the bands
    # as a GEMM, this entry point keeps the per-term kernels -- equal to FP64
    # rounding, not bit for bit.
    (W.Shape(40, 2, 1200, 19, 3), 4, True, False, False),
]


@pytest.mark.parametrize("shape,seed,band_independent,indinv,bit_identical", CASES)
def test_static_scratch_matches_gpp_sigma_twice(shape, seed, band_independent, indinv,
                                                bit_identical):
    from gppsigma import ops
    lib = capi.load()
    d = ops.DeviceInputs.from_host(_inputs(shape, seed, band_independent, indinv))
    assert (d.wx_stride == 0) == band_independent
    p = ops.problem_struct(d, "fp64", "complex_seq", 1.0)
    stream = torch.cuda.current_stream().cuda_stream
    o_ref, ref_ach, ref_asx = _outputs(shape.nw)
    capi.check(lib.gpp_sigma(C.byref(p), C.byref(o_ref), stream), "gpp_sigma")
    for _ in range(2):
        o, ach, asx = _outputs(shape.nw)
        capi.check(lib.gpp_sigma_static_scratch(C.byref(p), C.byref(o), stream),
                   "gpp_sigma_static_scratch")
        torch.cuda.synchronize()
        if bit_identical:
            assert torch.equal(torch.view_as_real(ach), torch.view_as_real(ref_ach))
            assert torch.equal(torch.view_as_real(asx), torch.view_as_real(ref_asx))
        assert rel_err(ach.cpu().numpy(), ref_ach.cpu().numpy()) <= FP64_TOL
        assert rel_err(asx.cpu().numpy(), ref_asx.cpu().numpy()) <= FP64_TOL


def test_static_scratch_applies_gpp_sigma_grid_limits():
    """More occupied bands than one launch's grid.y holds: rejected as
    unsupported before any launch, like gpp_sigma (no device pointer is read)."""
    lib = capi.load()
    p = capi.GppProblem()
    p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nw = 70000, 70000, 1, 1, 1
    p.aqsmtemp = p.aqsntemp = p.I_eps_array = p.wtilde_array = 0x1000
    p.vcoul = p.inv_igp_index = p.wx_array = 0x1000
    o = capi.GppOutputs()
    o.achtemp = o.asxtemp = 0x1000
    assert lib.gpp_sigma_static_scratch(C.byref(p), C.byref(o), None) == capi.GPP_ERR_UNSUPPORTED
    assert b"occupied bands" in lib.gpp_last_error_message()
    assert lib.gpp_sigma(C.byref(p), C.byref(o), None) == capi.GPP_ERR_UNSUPPORTED


def test_static_scratch_rejects_oversized_problem():
    lib = capi.load()
    p = capi.GppProblem()
    # 65535 band tiles x 1000 row tiles of partials: far beyond the 8 MiB buffer.
    p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nw = 4 * 65535, 0, 16, 2000, 3
    p.aqsmtemp = p.aqsntemp = p.I_eps_array = p.wtilde_array = 0x1000
    p.vcoul = p.inv_igp_index = p.wx_array = 0x1000
    o = capi.GppOutputs()
    o.achtemp = o.asxtemp = 0x1000
    st = lib.gpp_sigma_static_scratch(C.byref(p), C.byref(o), None)
    assert st == capi.GPP_ERR_UNSUPPORTED
    assert b"static buffer" in lib.gpp_last_error_message()
    p.precision = capi.PRECISION["mixed"]
    p.number_bands = 4
    assert lib.gpp_sigma_static_scratch(C.byref(p), C.byref(o), None) == capi.GPP_ERR_UNSUPPORTED

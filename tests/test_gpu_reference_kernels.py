"""The reference's own CUDA kernels (GPPComplex.cu, loaded from the cubin
that oracle/build_oracle.py compiles from the reference sources) on the same
device inputs as the new drop-in entry points: same achtemp within the FP64
tolerance.  The shape checks that keep those kernels in bounds run on the
CPU."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO, rel_err

sys.path.insert(0, os.path.join(REPO, "oracle"))
import ref_gpu  # noqa: E402

FP64_TOL = 1e-12


@pytest.mark.parametrize("args", [
    (64, 2, 4095, 64, 3, 0),   # odd ncouls: the reference reads past inv_igp_index
    (64, 2, 32, 64, 3, 0),     # ncouls <= 32: unguarded column reads
    (64, 2, 4096, 63, 3, 0),   # odd ngpown: the reference skips the last row
    (64, 2, 4096, 64, 5, 0),   # the reference computes exactly 3 frequencies
    (64, 2, 4096, 64, 3, -1),  # negative G' index
])
def test_shapes_outside_the_reference_kernels_bounds_are_refused(args):
    with pytest.raises(ValueError):
        ref_gpu.check_shape(*args)
    ref_gpu.check_shape(64, 2, 4096, 64, 3, 0)


@pytest.mark.gpu
def test_reference_gpu_kernels_agree_with_the_dropin_entry_points():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.exists(ref_gpu.CUBIN):
        pytest.skip("reference cubin not built (needs the reference sources)")
    from gppsigma import build, ops, workload as W
    build.build()
    shape = W.Shape(64, 2, 4096, 64, 3, near_pole=0.01)
    d = ref_gpu.band_independent(ops.device_inputs(shape, 77))
    ref_gpu.check_shape(d.number_bands, d.nvband, d.ncouls, d.ngpown, d.nw,
                        int(d.inv_igp_index.min().item()))
    ref = ref_gpu.RefKernels()
    stream = torch.cuda.current_stream().cuda_stream
    a = ref_gpu.zeroed_outputs(d.number_bands)
    ref.run(d, a, stream)
    b = ref_gpu.zeroed_outputs(d.number_bands)
    ops.d_till_nvband(d.nvband, d.ngpown, d.ncouls, d.inv_igp_index, d.wx_array, d.wtilde_array,
                      d.aqsmtemp, d.aqsntemp, d.I_eps_array, b["asxtemp"], d.vcoul,
                      b["acht_n1_loc"], b["achtemp_re"], b["achtemp_im"], 1.0)
    ops.d_noFlagOCCSolver(d.number_bands, d.nvband, d.ngpown, d.ncouls, d.inv_igp_index,
                          d.wx_array, d.wtilde_array, d.aqsmtemp, d.aqsntemp, d.I_eps_array,
                          d.vcoul, b["achtemp_re"], b["achtemp_im"], b["acht_n1_loc"])
    torch.cuda.synchronize()
    ops.wait()
    ach = lambda o: (o["achtemp_re"] + 1j * o["achtemp_im"]).cpu().numpy()
    # asxtemp and acht_n1_loc are summed without atomics in the reference
    # kernels (GPPComplex.cu:238,247,372), so only achtemp is comparable.
    assert np.all(np.isfinite(ach(a)))
    assert rel_err(ach(b), ach(a)) <= FP64_TOL


@pytest.mark.gpu
def test_reference_unified_memory_kernel_agrees_without_occupied_bands():
    """gppCuda.cu's call_compute (one thread per (n1, G' row)); its occupied
    bands carry sums across frequencies, so the comparison has nvband = 0."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.exists(ref_gpu.CUBIN_UNIFIED):
        pytest.skip("reference cubin not built (needs the reference sources)")
    from gppsigma import build, ops, workload as W
    build.build()
    shape = W.Shape(64, 0, 4096, 64, 3, near_pole=0.01)  # 64 * 64 pairs: 16 full blocks
    d = ref_gpu.band_independent(ops.device_inputs(shape, 78))
    ref_gpu.check_shape(d.number_bands, d.nvband, d.ncouls, d.ngpown, d.nw,
                        int(d.inv_igp_index.min().item()))
    uni = ref_gpu.UnifiedKernel()
    a = ref_gpu.zeroed_outputs(d.number_bands)
    uni.run(d, a, torch.cuda.current_stream().cuda_stream)
    b = ref_gpu.zeroed_outputs(d.number_bands)
    ops.d_noFlagOCCSolver(d.number_bands, d.nvband, d.ngpown, d.ncouls, d.inv_igp_index,
                          d.wx_array, d.wtilde_array, d.aqsmtemp, d.aqsntemp, d.I_eps_array,
                          d.vcoul, b["achtemp_re"], b["achtemp_im"], b["acht_n1_loc"])
    torch.cuda.synchronize()
    ops.wait()
    got = a["achtemp"].cpu().numpy()
    want = (b["achtemp_re"] + 1j * b["achtemp_im"]).cpu().numpy()
    assert np.all(np.isfinite(got))
    assert rel_err(want, got) <= FP64_TOL

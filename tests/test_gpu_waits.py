"""The failure path of the mixed kernels' bounded shared-memory pipeline
waits, exercised without a fault: a self-test block waits on a barrier that
nothing completes, gives up after a bounded number of polls and records the
timeout; the host sees GPP_ERR_DEVICE_TIMEOUT once and the context keeps
working."""
import time

import pytest

from conftest import rel_err
from gppsigma import build, capi, workload as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()
    capi.load()


def test_a_wait_that_runs_out_is_reported_and_the_context_survives():
    from gppsigma import ops
    lib = capi.load()
    inp = W.make_inputs(W.Shape(10, 2, 1000, 17, 3), 81)
    d = ops.DeviceInputs.from_host(inp)
    before = ops.sigma(d, "mixed")
    ops.wait()
    t0 = time.perf_counter()
    stream = torch.cuda.current_stream().cuda_stream
    capi.check(lib.gpp_selftest_wait_timeout(1 << 12, stream), "gpp_selftest_wait_timeout")
    with pytest.raises(capi.GppError) as err:
        ops.wait()
    assert err.value.status == capi.GPP_ERR_DEVICE_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
    ops.wait()  # reported once, then cleared
    after = ops.sigma(d, "mixed")
    ops.wait()
    assert rel_err(after.achtemp.cpu().numpy(), before.achtemp.cpu().numpy()) == 0.0


def test_self_test_rejects_out_of_range_polls():
    lib = capi.load()
    assert lib.gpp_selftest_wait_timeout(0, None) == capi.GPP_ERR_INVALID_ARGUMENT
    assert lib.gpp_selftest_wait_timeout(1 << 23, None) == capi.GPP_ERR_INVALID_ARGUMENT

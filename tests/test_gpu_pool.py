"""The library draws its workspace from a memory pool of its own: the caller's
default CUDA memory pool, and its release threshold, are left as they were
(a caller's own cudaMallocAsync keeps returning memory to the system)."""
import ctypes as C

import pytest

from gppsigma import build, capi, workload as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CU_MEMPOOL_ATTR_RELEASE_THRESHOLD = 4  # cuda.h, CUmemPool_attribute


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()
    capi.load()


def _default_pool_threshold() -> int:
    cu = C.CDLL("libcuda.so.1")
    assert cu.cuInit(0) == 0
    dev = C.c_int()
    assert cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
    pool = C.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    val = C.c_uint64()
    assert cu.cuMemPoolGetAttribute(pool, CU_MEMPOOL_ATTR_RELEASE_THRESHOLD, C.byref(val)) == 0
    return val.value


def test_default_pool_is_left_untouched():
    from gppsigma import ops
    torch.cuda.init()
    before = _default_pool_threshold()
    d = ops.DeviceInputs.from_host(W.make_inputs(W.Shape(12, 2, 700, 9, 3, near_pole=0.02), 5))
    for precision in ("fp64", "mixed"):
        ops.sigma(d, precision, acht_n1=True, achstemp=True)
    ops.wait()
    assert _default_pool_threshold() == before

"""Randomised small shapes through both CUDA paths: ragged ncouls, odd and
tiny ngpown, every frequency-chunk remainder, occupied-band counts from none
to all, near-pole wtilde, clamped G' indices and both semantics.  The shapes
come from a fixed seed, so a failure names a reproducible case.

Norm-wise tolerances (max |got - want| over max |want|, per output array):
with random inputs some components nearly cancel, and a per-component
relative bound would measure the cancellation rather than the kernel.
FP64 vs the oracle 1e-12; mixed vs the FP64 kernel 1e-8."""
import numpy as np
import pytest

from gppsigma import build, capi, workload as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FP64_TOL = 1e-12
MIXED_TOL = 1e-8


def shapes(n=48, seed=2026):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nw = int(rng.choice([1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 16, 33]))
        nb = int(rng.integers(1, 33 if nw <= 9 else 12))
        nv = int(rng.integers(0, nb + 1))
        nc = int(rng.integers(1, 2500))
        ng = min(int(rng.integers(1, 40 if nw <= 9 else 12)), nc)  # ng distinct columns
        near = float(rng.choice([0.0, 0.05]))
        over = int(rng.integers(0, 3)) if ng > 3 else 0
        sem = "kerseq" if i % 3 == 2 else "complex_seq"
        out.append((W.Shape(nb, nv, nc, ng, nw, near_pole=near, igp_overflow=over), sem,
                    1000 + i))
    return out


def normwise(got, want):
    got, want = np.asarray(got), np.asarray(want)
    scale = np.max(np.abs(want)) if want.size else 0.0
    return float(np.max(np.abs(got - want)) / scale) if scale > 0 else float(np.max(np.abs(got)))


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()
    capi.load()


@pytest.mark.parametrize("shape,semantics,seed", shapes(),
                         ids=lambda v: (f"nb{v.number_bands}-nv{v.nvband}-nc{v.ncouls}-"
                                        f"ng{v.ngpown}-nw{v.nw}-np{v.near_pole}-ov{v.igp_overflow}")
                         if isinstance(v, W.Shape) else str(v))
def test_random_shape_both_paths(shape, semantics, seed):
    import oracle_py
    from gppsigma import ops
    inp = W.make_inputs(shape, seed)
    want = oracle_py.run(inp, semantics)
    d = ops.DeviceInputs.from_host(inp)
    n1 = shape.nw >= 3
    r64 = ops.sigma(d, "fp64", semantics, acht_n1=n1, achstemp=True)
    rmx = ops.sigma(d, "mixed", semantics, acht_n1=n1, achstemp=True)
    ops.wait()
    for key in ("achtemp", "asxtemp"):
        g64 = getattr(r64, key).cpu().numpy()
        gmx = getattr(rmx, key).cpu().numpy()
        assert normwise(g64, want[key]) <= FP64_TOL, key
        assert normwise(gmx, g64) <= MIXED_TOL, key
    assert normwise(r64.achstemp.cpu().numpy(), want["achstemp"]) <= FP64_TOL
    if n1:
        g64 = r64.acht_n1_loc.cpu().numpy()
        assert normwise(g64, want["acht_n1_loc"]) <= FP64_TOL
        assert normwise(rmx.acht_n1_loc.cpu().numpy(), g64) <= MIXED_TOL

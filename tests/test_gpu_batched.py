"""Batched states in one persistent launch: every state's result equals the
one-state call on the same inputs (same tiles, same reduction tree), for FP64
and mixed precision, one-shot and through a reusable plan replayed from a
CUDA graph (including after the inputs change in place)."""
import ctypes as C

import numpy as np
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


def _states(n=5, nw=3, seed=3):
    from gppsigma import ops
    shapes = W.batched_shapes(n, seed, scale=0.05)
    shapes = [W.Shape(s.number_bands, s.nvband, s.ncouls, s.ngpown, nw, near_pole=0.01)
              for s in shapes]
    return [ops.DeviceInputs.from_host(W.make_inputs(s, seed + i)) for i, s in enumerate(shapes)]


def _arrays(devs, precision, with_n1):
    from gppsigma import ops
    probs = (capi.GppProblem * len(devs))()
    outs = (capi.GppOutputs * len(devs))()
    keep = []
    for i, d in enumerate(devs):
        probs[i] = ops.problem_struct(d, precision, "complex_seq", 1.0)
        a = torch.full((d.nw,), float("nan"), dtype=torch.complex128, device="cuda")
        x = torch.full((d.nw,), float("nan"), dtype=torch.complex128, device="cuda")
        n1 = torch.zeros(d.number_bands, dtype=torch.complex128, device="cuda") if with_n1 else None
        outs[i].achtemp, outs[i].asxtemp = a.data_ptr(), x.data_ptr()
        outs[i].acht_n1_loc = n1.data_ptr() if n1 is not None else None
        keep.append((a, x, n1))
    return probs, outs, keep


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_one_shot_batch_equals_per_state_calls(precision):
    from gppsigma import ops
    lib = capi.load()
    devs = _states()
    probs, outs, keep = _arrays(devs, precision, with_n1=True)
    stream = torch.cuda.current_stream().cuda_stream
    capi.check(lib.gpp_sigma_batched(probs, outs, len(devs), stream), "gpp_sigma_batched")
    for d, (a, x, n1) in zip(devs, keep):
        ref = ops.sigma(d, precision, acht_n1=True)
        ops.wait()
        assert torch.equal(torch.view_as_real(a), torch.view_as_real(ref.achtemp))
        assert torch.equal(torch.view_as_real(x), torch.view_as_real(ref.asxtemp))
        assert torch.equal(torch.view_as_real(n1), torch.view_as_real(ref.acht_n1_loc))


def test_plan_replays_from_a_graph_and_sees_new_inputs():
    from gppsigma import ops
    lib = capi.load()
    devs = _states(4, seed=11)
    probs, outs, keep = _arrays(devs, "mixed", with_n1=False)
    plan = C.c_void_p()
    capi.check(lib.gpp_batch_create(C.byref(plan), probs, outs, len(devs)), "gpp_batch_create")
    try:
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            for _ in range(2):
                capi.check(lib.gpp_batch_run(plan, s.cuda_stream), "gpp_batch_run")
            s.synchronize()
            first = [torch.view_as_real(a).clone() for a, _, _ in keep]
            devs[1].wtilde_array.mul_(1.001)  # same addresses, new contents
            capi.check(lib.gpp_batch_run(plan, s.cuda_stream), "gpp_batch_run")
            s.synchronize()
        for i, (d, (a, x, _)) in enumerate(zip(devs, keep)):
            ref = ops.sigma(d, "mixed")
            ops.wait()
            assert torch.equal(torch.view_as_real(a), torch.view_as_real(ref.achtemp))
            if i != 1:
                assert torch.equal(torch.view_as_real(a), first[i])
            else:
                assert not torch.equal(torch.view_as_real(a), first[i])
    finally:
        lib.gpp_batch_destroy(plan)


def test_batch_rejects_mixed_nw():
    lib = capi.load()
    devs = _states(2)
    devs2 = _states(1, nw=2, seed=5)
    probs, outs, keep = _arrays(devs + devs2, "fp64", with_n1=False)
    st = lib.gpp_sigma_batched(probs, outs, 3, None)
    assert st == capi.GPP_ERR_UNSUPPORTED


def test_batch_follows_the_tuned_tile_shape():
    """With an 8-bands-per-block variant chosen for 3 frequencies (as
    gpp_autotune or gpp_set_variant would), the persistent kernel runs that
    tile shape too: every state's bits equal its one-state call under the
    same choice, and differ from the default shape's only by rounding."""
    from gppsigma import ops
    lib = capi.load()
    names = ops.variant_names()
    v8 = next(i for i, n in enumerate(names) if n.startswith("8 bands x 2 rows (8 warps)"))
    devs = _states()
    stream = torch.cuda.current_stream().cuda_stream
    try:
        capi.check(lib.gpp_set_variant(3, v8), "gpp_set_variant")
        probs, outs, keep = _arrays(devs, "mixed", with_n1=False)
        capi.check(lib.gpp_sigma_batched(probs, outs, len(devs), stream), "gpp_sigma_batched")
        for d, (a, x, _) in zip(devs, keep):
            ref = ops.sigma(d, "mixed")
            ops.wait()
            assert torch.equal(torch.view_as_real(a), torch.view_as_real(ref.achtemp))
            assert torch.equal(torch.view_as_real(x), torch.view_as_real(ref.asxtemp))
    finally:
        ops.set_variant(3, -1)
    for d, (a, x, _) in zip(devs, keep):
        base = ops.sigma(d, "mixed")
        ops.wait()
        assert rel_err(a.cpu().numpy(), base.achtemp.cpu().numpy()) <= 1e-10

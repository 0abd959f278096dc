"""The band-sum GEMM path of FP64 calls with band-independent frequencies:
the same sums as the per-term kernel and the oracle (achtemp, asxtemp,
acht_n1_loc, the static term), on ragged shapes, clamped G' indices,
near-pole wtilde, every frequency-chunk width and the overlapped host path;
with the GEMMs on the tensor cores (the default, mode 1) and on the FP64
pipe (mode 2)."""
import dataclasses

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


def band_independent(shape, seed):
    inp = W.make_inputs(shape, seed)
    inp.wx_array = inp.wx_array[:1].copy()  # one wx row for every band
    return inp


def sigma_with(mode, d, semantics, n1):
    from gppsigma import ops
    lib = capi.load()
    capi.check(lib.gpp_set_gemm_path(mode), "gemm path")
    try:
        r = ops.sigma(d, "fp64", semantics, acht_n1=n1, achstemp=True)
        ops.wait()
    finally:
        capi.check(lib.gpp_set_gemm_path(-1), "gemm path")
    return r


@pytest.mark.parametrize("shape,semantics", [
    (W.Shape(40, 2, 777, 13, 3, near_pole=0.05), "complex_seq"),
    (W.Shape(37, 0, 1000, 21, 1), "complex_seq"),
    (W.Shape(33, 5, 640, 8, 5, igp_overflow=2), "kerseq"),
    (W.Shape(64, 3, 2048, 64, 8, dw=0.25), "complex_seq"),
    (W.Shape(20, 4, 300, 1, 3), "kerseq"),
    (W.Shape(40, 2, 1, 1, 3), "complex_seq"),
    (W.Shape(6, 5, 35, 3, 2), "complex_seq"),
])
def test_gemm_path_equals_per_term_kernel_and_oracle(shape, semantics):
    import oracle_py
    from gppsigma import ops
    inp = band_independent(shape, 91)
    want = oracle_py.run(inp, semantics)
    d = ops.DeviceInputs.from_host(inp)
    assert d.wx_stride == 0
    n1 = shape.nw >= 3
    t = sigma_with(0, d, semantics, n1)
    for mode in (1, 2):
        g = sigma_with(mode, d, semantics, n1)
        for key in ("achtemp", "asxtemp", "achstemp"):
            a, b = getattr(g, key).cpu().numpy(), getattr(t, key).cpu().numpy()
            assert rel_err(a, want[key]) <= FP64_TOL, (mode, key)
            assert rel_err(a, b) <= FP64_TOL, (mode, key)
        if n1:
            a = g.acht_n1_loc.cpu().numpy()
            scale = np.max(np.abs(want["acht_n1_loc"]))
            assert np.max(np.abs(a - want["acht_n1_loc"])) <= FP64_TOL * scale, mode
            assert np.max(np.abs(a - t.acht_n1_loc.cpu().numpy())) <= FP64_TOL * scale, mode


def test_gemm_path_is_bit_reproducible_and_automatic_from_32_bands():
    from gppsigma import ops
    d = ops.DeviceInputs.from_host(band_independent(W.Shape(64, 2, 1500, 30, 3), 5))
    a = sigma_with(-1, d, "complex_seq", True)
    b = sigma_with(-1, d, "complex_seq", True)
    g = sigma_with(1, d, "complex_seq", True)
    for key in ("achtemp", "acht_n1_loc"):
        x, y, z = (getattr(r, key).cpu().numpy() for r in (a, b, g))
        assert np.array_equal(x, y) and np.array_equal(x, z), key
    lib = capi.load()
    assert lib.gpp_set_gemm_path(3) == capi.GPP_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("ngpown", [33, 4])
def test_gemm_path_through_the_host_pieces(ngpown):
    """gpp_sigma_host splits the G' rows into pieces; the GEMM path runs per
    piece and must give the device call's bits."""
    from gppsigma import ops
    inp = band_independent(W.Shape(48, 2, 900, ngpown, 3), 17)
    d = ops.DeviceInputs.from_host(inp)
    dev = sigma_with(1, d, "complex_seq", True)
    arrays = {k: getattr(inp, k) for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array",
                                           "vcoul", "inv_igp_index", "indinv", "wx_array")}
    lib = capi.load()
    capi.check(lib.gpp_set_gemm_path(1), "gemm path")
    try:
        with ops.HostContext() as ctx:
            host = ctx.sigma(arrays, inp.shape, "fp64", acht_n1=True)
    finally:
        capi.check(lib.gpp_set_gemm_path(-1), "gemm path")
    assert np.array_equal(host["achtemp"], dev.achtemp.cpu().numpy())
    assert np.array_equal(host["acht_n1_loc"], dev.acht_n1_loc.cpu().numpy())


MIXED_TOL = 1e-8


def mixed_with(mode, d, semantics, n1=False):
    from gppsigma import ops
    lib = capi.load()
    capi.check(lib.gpp_set_gemm_path(mode), "gemm path")
    try:
        r = ops.sigma(d, "mixed", semantics, acht_n1=n1, achstemp=False)
        ops.wait()
    finally:
        capi.check(lib.gpp_set_gemm_path(-1), "gemm path")
    return r


@pytest.mark.parametrize("shape,semantics", [
    (W.Shape(40, 2, 777, 13, 3, near_pole=0.05), "complex_seq"),
    (W.Shape(37, 0, 1000, 21, 1), "complex_seq"),
    (W.Shape(33, 5, 640, 8, 5, igp_overflow=2), "kerseq"),
    (W.Shape(64, 3, 2048, 64, 8, dw=0.25, near_pole=0.02), "complex_seq"),
    (W.Shape(20, 4, 300, 1, 3), "kerseq"),
    (W.Shape(150, 2, 4100, 70, 3, near_pole=0.01), "complex_seq"),
    (W.Shape(40, 2, 1, 1, 3), "complex_seq"),
    (W.Shape(6, 5, 35, 3, 2), "kerseq"),
    (W.Shape(300, 0, 4099, 5, 4, near_pole=0.05), "complex_seq"),
])
def test_mixed_gemm_path_within_1e8_of_fp64(shape, semantics):
    """The mixed-precision band-sum paths -- G from the tensor cores split
    into float-float (mode 1) and the float-float GEMM (mode 2) -- against
    the FP64 per-term kernel and the mixed per-term kernel."""
    from gppsigma import ops
    d = ops.DeviceInputs.from_host(band_independent(shape, 93))
    n1 = shape.nw >= 3
    f = sigma_with(0, d, semantics, n1)
    t = mixed_with(0, d, semantics, n1)
    for mode in (1, 2):
        m = mixed_with(mode, d, semantics, n1)
        for key in ("achtemp", "asxtemp"):
            a = getattr(m, key).cpu().numpy()
            assert rel_err(a, getattr(f, key).cpu().numpy()) <= MIXED_TOL, (mode, key)
            assert rel_err(a, getattr(t, key).cpu().numpy()) <= MIXED_TOL, (mode, key)
        if n1:  # per-band output (norm-wise: single bands cancel more than the sums)
            a, w = m.acht_n1_loc.cpu().numpy(), f.acht_n1_loc.cpu().numpy()
            assert np.max(np.abs(a - w)) <= MIXED_TOL * np.max(np.abs(w)), mode


def test_mixed_gemm_path_through_the_host_pieces():
    from gppsigma import ops
    inp = band_independent(W.Shape(48, 2, 900, 33, 3, near_pole=0.02), 19)
    d = ops.DeviceInputs.from_host(inp)
    dev = mixed_with(1, d, "complex_seq", True)
    arrays = {k: getattr(inp, k) for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array",
                                           "vcoul", "inv_igp_index", "indinv", "wx_array")}
    lib = capi.load()
    capi.check(lib.gpp_set_gemm_path(1), "gemm path")
    try:
        with ops.HostContext() as ctx:
            host = ctx.sigma(arrays, inp.shape, "mixed", acht_n1=True)
    finally:
        capi.check(lib.gpp_set_gemm_path(-1), "gemm path")
    assert np.array_equal(host["achtemp"], dev.achtemp.cpu().numpy())
    assert np.array_equal(host["asxtemp"], dev.asxtemp.cpu().numpy())
    assert np.array_equal(host["acht_n1_loc"], dev.acht_n1_loc.cpu().numpy())


@pytest.mark.parametrize("shape,semantics", [
    (W.Shape(40, 2, 777, 13, 3, near_pole=0.05), "complex_seq"),
    (W.Shape(33, 5, 640, 8, 4, igp_overflow=2), "kerseq"),
    (W.Shape(20, 3, 300, 9, 1), "complex_seq"),
    (W.Shape(16, 4, 513, 7, 2, near_pole=0.05), "kerseq"),
    (W.Shape(12, 1, 400, 5, 3), "complex_seq"),
    (W.Shape(24, 7, 256, 3, 8, dw=0.25), "complex_seq"),
])
def test_occupied_band_pairs_give_the_per_band_bits(shape, semantics, monkeypatch):
    """With one wx row for every band the FP64 occupied-band kernel solves
    each (row, column, frequency) once for a pair of bands.  Its sums must be
    the bits of one band per block: the same call with GPP_FLAG_MULTI=0, and
    the same wx replicated into one row per band (the per-band kernel)."""
    from gppsigma import ops
    inp = band_independent(shape, 23)
    rep = dataclasses.replace(inp, wx_array=np.repeat(inp.wx_array, shape.number_bands, axis=0))
    d = ops.DeviceInputs.from_host(inp)
    d_rep = ops.DeviceInputs.from_host(rep)
    assert d.wx_stride == 0 and d_rep.wx_stride == shape.nw
    n1 = shape.nw >= 3
    pair = sigma_with(0, d, semantics, n1)
    replicated = sigma_with(0, d_rep, semantics, n1)
    monkeypatch.setenv("GPP_FLAG_MULTI", "0")
    single = sigma_with(0, d, semantics, n1)
    keys = ("achtemp", "asxtemp") + (("acht_n1_loc",) if n1 else ())
    for key in keys:
        a = getattr(pair, key).cpu().numpy()
        assert np.array_equal(a, getattr(single, key).cpu().numpy()), key
        assert np.array_equal(a, getattr(replicated, key).cpu().numpy()), key


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("shape,semantics", [
    (W.Shape(48, 2, 1500, 301, 3, near_pole=0.05), "complex_seq"),
    (W.Shape(40, 5, 900, 37, 4), "kerseq"),
    (W.Shape(36, 3, 700, 19, 8, dw=0.25), "complex_seq"),
])
def test_occupied_band_grid_beside_the_tensor_gemm_keeps_the_bits(precision, shape, semantics,
                                                                   monkeypatch):
    """Beside the tensor-core GEMM the occupied-band kernel may run as a
    persistent grid taking (row tile, band group, chunk) items from a work
    counter (the FP64 default), one block per row tile (the float-float
    default) or before the GEMM on the same stream (GPP_OVERLAP_TENSOR_GEMM=0);
    every item is computed and written the same way and the partials are
    reduced in one fixed order, so every choice gives the same bits."""
    from gppsigma import ops
    d = ops.DeviceInputs.from_host(band_independent(shape, 31))
    lib = capi.load()

    def run():
        capi.check(lib.gpp_set_gemm_path(1), "gemm path")
        try:
            r = ops.sigma(d, precision, semantics, acht_n1=True)
            ops.wait()
        finally:
            capi.check(lib.gpp_set_gemm_path(-1), "gemm path")
        return {k: getattr(r, k).cpu().numpy() for k in ("achtemp", "asxtemp", "acht_n1_loc")}

    base = run()
    for env in ({"GPP_FLAG_BLOCKS_PER_SM": "0"}, {"GPP_FLAG_BLOCKS_PER_SM": "1"},
                {"GPP_FLAG_BLOCKS_PER_SM": "2"}, {"GPP_OVERLAP_TENSOR_GEMM": "0"}):
        with monkeypatch.context() as m:
            for k, v in env.items():
                m.setenv(k, v)
            got = run()
        for key, want in base.items():
            assert np.array_equal(got[key], want), (env, key)

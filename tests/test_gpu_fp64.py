"""FP64 CUDA path against the reference: golden fixtures produced by the
reference's own functions, its README known answers, the reference-signature
entry points, determinism, device-side fault reporting and the host path."""
import dataclasses
import os
import subprocess

import numpy as np
import pytest

from conftest import case_inputs, load_golden, rel_err, unhex
from gppsigma import build, capi, workload as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FP64_TOL = 1e-12  # per real/imaginary component, relative
CASES = load_golden()


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()
    capi.load()


def ops():
    from gppsigma import ops as o
    return o


def check_case(res, case, tol=FP64_TOL):
    assert rel_err(res.achtemp.cpu().numpy(), unhex(case["achtemp"])) <= tol
    assert rel_err(res.asxtemp.cpu().numpy(), unhex(case["asxtemp"])) <= tol
    if res.achstemp is not None:
        assert rel_err(res.achstemp.cpu().numpy(), unhex(case["achstemp"])) <= tol
    if res.acht_n1_loc is not None and case["acht_n1_loc"] is not None:
        want = unhex(case["acht_n1_loc"])
        got = res.acht_n1_loc.cpu().numpy()
        scale = max(np.max(np.abs(want)), 1e-300)
        assert np.max(np.abs(got - want)) <= tol * scale


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_fp64_matches_reference_fixture(case):
    o = ops()
    inp = case_inputs(case)
    d = o.DeviceInputs.from_host(inp)
    want_n1 = inp.shape.nw >= 3
    res = o.sigma(d, "fp64", case["semantics"], acht_n1=want_n1, achstemp=True)
    o.wait()
    check_case(res, case)


def test_readme_known_answer_through_reference_driver():
    """The reference's CUDA call sequence (gppCudaVer.cpp:389-399) on the
    README small case, run by gpp_driver.ex against libgpp_gb300.so."""
    build.build()
    out = subprocess.run([build.DRIVER, "512", "2", "800", "20"], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    case = next(c for c in CASES if c["name"] == "ramp_512_2_800_20")
    got = []
    for line in out.stdout.splitlines():
        if line.startswith("achtemp["):
            re_s, im_s = line.split("= (")[1].rstrip(")").split(",")
            got.append(complex(float(re_s), float(im_s)))
    readme = [complex(*map(float, s.strip("()").split(","))) for s in case["readme_achtemp"]]
    assert len(got) == 3
    assert rel_err(got, readme) <= 1e-13  # README rounds to 15 digits
    assert rel_err(got, unhex(case["achtemp"])) <= FP64_TOL


def test_reference_entry_points_accumulate_like_the_reference():
    o = ops()
    inp = W.make_inputs(W.Shape(10, 3, 700, 11, 3), 31)
    inp.wx_array = inp.wx_array[:1].copy()  # band-independent wx, as the reference
    import oracle_py
    want = oracle_py.run(inp, "complex_seq")
    d = o.DeviceInputs.from_host(inp)
    s = inp.shape
    re_ = torch.zeros(3, dtype=torch.float64, device="cuda")
    im_ = torch.zeros(3, dtype=torch.float64, device="cuda")
    asx = torch.zeros(3, dtype=torch.complex128, device="cuda")
    n1 = torch.zeros(s.number_bands, dtype=torch.complex128, device="cuda")
    for _ in range(2):  # the reference adds into its outputs; two calls double them
        o.d_till_nvband(s.nvband, s.ngpown, s.ncouls, d.inv_igp_index, d.wx_array, d.wtilde_array,
                        d.aqsmtemp, d.aqsntemp, d.I_eps_array, asx, d.vcoul, n1, re_, im_, 1.0)
        o.d_noFlagOCCSolver(s.number_bands, s.nvband, s.ngpown, s.ncouls, d.inv_igp_index,
                            d.wx_array, d.wtilde_array, d.aqsmtemp, d.aqsntemp, d.I_eps_array,
                            d.vcoul, re_, im_, n1)
    o.wait()
    ach = (re_ + 1j * im_).cpu().numpy() / 2
    assert rel_err(ach, want["achtemp"]) <= FP64_TOL
    assert rel_err(asx.cpu().numpy() / 2, want["asxtemp"]) <= FP64_TOL
    assert np.max(np.abs(n1.cpu().numpy() / 2 - want["acht_n1_loc"])) <= FP64_TOL * np.max(np.abs(want["acht_n1_loc"]))

    # gppKernelGPU: every band unoccupied.
    inp0 = W.Inputs(W.Shape(10, 0, 700, 11, 3), inp.seed, inp.aqsmtemp, inp.aqsntemp,
                    inp.I_eps_array, inp.wtilde_array, inp.vcoul, inp.inv_igp_index, inp.indinv,
                    inp.wx_array)
    want0 = oracle_py.run(inp0, "complex_seq")
    re0 = torch.zeros(3, dtype=torch.float64, device="cuda")
    im0 = torch.zeros(3, dtype=torch.float64, device="cuda")
    o.gppKernelGPU(d.wtilde_array, d.aqsntemp, d.aqsmtemp, d.I_eps_array, s.ncouls, s.ngpown,
                   s.number_bands, d.wx_array, re0, im0, d.vcoul, 0, 3, d.indinv, d.inv_igp_index)
    achs_re = torch.zeros(1, dtype=torch.float64, device="cuda")
    achs_im = torch.zeros(1, dtype=torch.float64, device="cuda")
    o.d_reduce_achstemp(s.number_bands, d.inv_igp_index, s.ncouls, d.aqsmtemp, d.aqsntemp,
                        d.I_eps_array, achs_re, achs_im, s.ngpown, d.vcoul)
    # The C ABI's complex-destination form gives the same bits.
    achs = torch.zeros(1, dtype=torch.complex128, device="cuda")
    capi.check(capi.load().gpp_reduce_achstemp(
        s.number_bands, d.inv_igp_index.data_ptr(), s.ncouls, d.aqsmtemp.data_ptr(),
        d.aqsntemp.data_ptr(), d.I_eps_array.data_ptr(), achs.data_ptr(), s.ngpown,
        d.vcoul.data_ptr()), "gpp_reduce_achstemp")
    o.wait()
    assert rel_err((re0 + 1j * im0).cpu().numpy(), want0["achtemp"]) <= FP64_TOL
    assert rel_err((achs_re + 1j * achs_im).cpu().numpy(), want["achstemp"]) <= FP64_TOL
    assert torch.equal(torch.view_as_real(achs)[0], torch.stack([achs_re[0], achs_im[0]]))


def test_bit_reproducible_run_to_run():
    o = ops()
    d = o.DeviceInputs.from_host(W.make_inputs(W.Shape(64, 4, 4096, 256, 3), 11))
    a = o.sigma(d, "fp64", acht_n1=True, achstemp=True)
    b = o.sigma(d, "fp64", acht_n1=True, achstemp=True)
    o.wait()
    for x, y in ((a.achtemp, b.achtemp), (a.asxtemp, b.asxtemp), (a.acht_n1_loc, b.acht_n1_loc),
                 (a.achstemp, b.achstemp)):
        assert torch.equal(torch.view_as_real(x), torch.view_as_real(y))


def test_device_side_index_fault_is_reported_then_cleared():
    o = ops()
    inp = W.make_inputs(W.Shape(6, 2, 300, 8, 3), 41)
    inp.inv_igp_index[2] = -5
    d = o.DeviceInputs.from_host(inp)
    o.sigma(d, "fp64")
    with pytest.raises(capi.GppError) as ei:
        o.wait()
    assert ei.value.status == capi.GPP_ERR_BAD_INDEX
    o.wait()  # the fault word was cleared
    d.indinv[0] = 10**6  # indinv out of range
    inp.inv_igp_index[2] = 0
    d.inv_igp_index.copy_(torch.from_numpy(inp.inv_igp_index))
    o.sigma(d, "fp64")
    with pytest.raises(capi.GppError):
        o.wait()


@pytest.mark.parametrize("memory", ["pageable", "pinned"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ngpown", [20, 3, 33])
def test_host_path_equals_device_path(precision, ngpown, memory):
    """The host path moves the G' rows in pieces and starts each piece's
    kernels when its rows land; the bits must equal one device-path call.
    Pinned arrays are pulled by the SMs (those whose size is not a multiple
    of 16 bytes -- inv_igp_index at 3 and 33 rows -- go through the copy
    engine beside them); pageable ones through the copy engine."""
    o = ops()
    inp = W.make_inputs(W.Shape(12, 3, 1000, ngpown, 3, near_pole=0.05), 51)
    d = o.DeviceInputs.from_host(inp)
    dev = o.sigma(d, precision, acht_n1=True, achstemp=True)
    o.wait()
    keep = {}
    arrays = {}
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul", "inv_igp_index",
              "indinv", "wx_array"):
        a = np.ascontiguousarray(getattr(inp, k))
        if memory == "pinned":
            keep[k] = torch.from_numpy(a).pin_memory()
            a = keep[k].numpy()
        arrays[k] = a
    with o.HostContext() as ctx:
        with pytest.raises(capi.GppError):
            ctx.last_timing()  # nothing timed yet
        host = ctx.sigma(arrays, inp.shape, precision, acht_n1=True, achstemp=True)
        host2 = ctx.sigma(arrays, inp.shape, precision, acht_n1=True, achstemp=True)
        t = ctx.last_timing()
    assert t["h2d_ms"] > 0 and t["compute_ms"] > 0 and t["d2h_ms"] >= 0
    for k in ("achtemp", "asxtemp", "acht_n1_loc", "achstemp"):
        np.testing.assert_array_equal(host[k], getattr(dev, k).cpu().numpy())
        np.testing.assert_array_equal(host[k], host2[k])


def test_non_default_stream():
    o = ops()
    inp = W.make_inputs(W.Shape(9, 2, 800, 15, 3), 61)
    d = o.DeviceInputs.from_host(inp)
    ref = o.sigma(d, "fp64")
    o.wait()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        got = o.sigma(d, "fp64")
        o.wait()
    assert torch.equal(torch.view_as_real(ref.achtemp), torch.view_as_real(got.achtemp))


def _slice_bands(inp, a, b):
    s = inp.shape
    nv = max(0, min(s.nvband, b) - a)
    shp = W.Shape(b - a, nv, s.ncouls, s.ngpown, s.nw, s.dw)
    return W.Inputs(shp, inp.seed, inp.aqsmtemp[a:b], inp.aqsntemp[a:b], inp.I_eps_array,
                    inp.wtilde_array, inp.vcoul, inp.inv_igp_index, inp.indinv, inp.wx_array[a:b])


def test_production_shape_band_partition_and_oracle_subset():
    """Full production shape (512 bands, ncouls 32768, ngpown 1638): the sum
    over a band partition equals the one-call result (linearity), and a band
    subset with both occupied and unoccupied bands matches the oracle."""
    o = ops()
    import oracle_py
    inp = W.make_inputs(W.CONFIGS["production"], 20240607)
    d = o.DeviceInputs.from_host(inp)
    full = o.sigma(d, "fp64")
    o.wait()
    total = np.zeros(3, np.complex128)
    asx = np.zeros(3, np.complex128)
    for a, b in ((0, 100), (100, 300), (300, 512)):
        r = o.sigma(o.DeviceInputs.from_host(_slice_bands(inp, a, b)), "fp64")
        o.wait()
        total += r.achtemp.cpu().numpy()
        asx += r.asxtemp.cpu().numpy()
    assert rel_err(total, full.achtemp.cpu().numpy()) <= 1e-11
    assert rel_err(asx, full.asxtemp.cpu().numpy()) <= 1e-11
    sub = _slice_bands(inp, 0, 4)
    r = o.sigma(o.DeviceInputs.from_host(sub), "fp64")
    o.wait()
    want = oracle_py.run(sub, "complex_seq", nthreads=max(1, os.cpu_count() or 1))
    assert rel_err(r.achtemp.cpu().numpy(), want["achtemp"]) <= FP64_TOL
    assert rel_err(r.asxtemp.cpu().numpy(), want["asxtemp"]) <= FP64_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_row_shards_add_up_to_the_full_call(precision):
    """A state sharded by G' rows (one slice per rank in a multi-GPU run):
    the slices' sums add up to the one-call sums."""
    from gppsigma import dist as gd
    o = ops()
    inp = W.make_inputs(W.Shape(20, 2, 1500, 37, 3, near_pole=0.02), 71)
    d = o.DeviceInputs.from_host(inp)
    full = o.sigma(d, precision, achstemp=True)
    parts = [o.sigma(d.rows(*gd.row_range(37, r, 3)), precision, achstemp=True) for r in range(3)]
    o.wait()
    for key in ("achtemp", "asxtemp", "achstemp"):
        total = sum(getattr(p_, key).cpu().numpy() for p_ in parts)
        assert rel_err(total, getattr(full, key).cpu().numpy()) <= 1e-12, key


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_indinv_remaps_the_clamped_igp(precision):
    """A non-identity indinv (GPPComplex.h:304) remaps igp = indinv[min(inv_igp_index,
    ncouls-1)]: the same bits as the identity indinv with that map folded into
    inv_igp_index."""
    o = ops()
    shape = W.Shape(12, 2, 800, 21, 3, near_pole=0.02, igp_overflow=3)
    inp = W.make_inputs(shape, 91)
    perm = np.random.default_rng(3).permutation(shape.ncouls).astype(np.int32)
    a_in = dataclasses.replace(inp, indinv=perm)
    folded = perm[np.minimum(inp.inv_igp_index, shape.ncouls - 1)].astype(np.int32)
    b_in = dataclasses.replace(inp, inv_igp_index=folded)
    a = o.sigma(o.DeviceInputs.from_host(a_in), precision, acht_n1=True, achstemp=True)
    b = o.sigma(o.DeviceInputs.from_host(b_in), precision, acht_n1=True, achstemp=True)
    o.wait()
    for key in ("achtemp", "asxtemp", "acht_n1_loc", "achstemp"):
        assert torch.equal(torch.view_as_real(getattr(a, key)), torch.view_as_real(getattr(b, key))), key


def test_unmodified_reference_driver_runs_mixed_from_the_environment():
    """GPP_DROPIN_PRECISION=mixed makes the reference's own call sequence
    (gpp_driver.ex) use the float-float kernels: the README known answer
    within 1e-8."""
    build.build()
    env = dict(os.environ, GPP_DROPIN_PRECISION="mixed")
    out = subprocess.run([build.DRIVER, "512", "2", "800", "20"], capture_output=True, text=True,
                         timeout=120, env=env)
    assert out.returncode == 0, out.stderr
    case = next(c for c in CASES if c["name"] == "ramp_512_2_800_20")
    got = []
    for line in out.stdout.splitlines():
        if line.startswith("achtemp["):
            re_s, im_s = line.split("= (")[1].rstrip(")").split(",")
            got.append(complex(float(re_s), float(im_s)))
    assert len(got) == 3
    assert rel_err(got, unhex(case["achtemp"])) <= 1e-8

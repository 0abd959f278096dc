"""Seeded workload generator: reproducibility and distributions."""
import numpy as np

from gppsigma import workload as W


def test_uniform_independent_of_chunking(monkeypatch):
    a = W.uniform(5, 3, 10000, -0.5, 0.5)
    monkeypatch.setattr(W, "_CHUNK", 777)
    b = W.uniform(5, 3, 10000, -0.5, 0.5)
    np.testing.assert_array_equal(a, b)
    assert a.min() >= -0.5 and a.max() < 0.5


def test_distributions_and_index_set():
    s = W.Shape(64, 2, 4096, 200, 3)
    inp = W.make_inputs(s, 1)
    assert inp.aqsmtemp.shape == (64, 4096) and inp.I_eps_array.shape == (200, 4096)
    assert np.all(np.abs(inp.aqsmtemp.real) <= 0.5) and np.all(np.abs(inp.I_eps_array.imag) <= 0.5)
    assert inp.wtilde_array.real.min() >= 0.5 and inp.wtilde_array.real.max() < 2.0
    assert np.all(np.abs(inp.wtilde_array.imag) <= 0.05)
    assert inp.vcoul.min() >= 0.1 and inp.vcoul.max() < 1.0
    igp = inp.inv_igp_index
    assert len(np.unique(igp)) == 200 and np.all(np.diff(igp) > 0) and igp.max() < 4096
    e_n1 = 10.0 + 1.0 - inp.wx_array[:, 0]
    assert e_n1.min() >= 0.0 and e_n1.max() <= 20.0
    np.testing.assert_allclose(np.diff(inp.wx_array, axis=1), 1.0)
    assert np.array_equal(inp.indinv, np.arange(4096))


def test_same_seed_same_digest_new_seed_new_digest():
    s = W.Shape(8, 2, 256, 8, 3)
    assert W.make_inputs(s, 3).digest() == W.make_inputs(s, 3).digest()
    assert W.make_inputs(s, 3).digest() != W.make_inputs(s, 4).digest()


def test_near_pole_entries_sit_next_to_a_frequency():
    s = W.Shape(16, 2, 2048, 32, 3, near_pole=0.01)
    inp = W.make_inputs(s, 2)
    wt = inp.wtilde_array.ravel()
    d = np.min(np.abs(wt[:, None] - inp.wx_array.ravel()[None, :]), axis=1)
    frac = np.mean(d < 1e-4)
    assert 0.005 < frac < 0.02


def test_ramp_inputs_are_the_reference_ramp():
    inp = W.ramp_inputs(512, 2, 800, 20)
    assert inp.shape.ngpown == 40
    assert inp.aqsntemp[3, 5] == 4.0 + 4.0j and inp.I_eps_array[2, 7] == 4.5 + 4.5j
    assert list(inp.inv_igp_index[:3]) == [20, 40, 60] and inp.inv_igp_index[-1] == 800
    np.testing.assert_array_equal(inp.wx_array[0], [3.0, 4.0, 5.0])


def test_batched_shapes_ranges():
    shapes = W.batched_shapes(64, 5)
    assert len(shapes) == 64
    for s in shapes:
        assert 256 <= s.number_bands <= 2048 and 8192 <= s.ncouls <= 65536
        assert 2 <= s.nvband <= 8 and s.ngpown == s.ncouls // 20 and s.nw == 3


def test_device_generator_matches_host_generator():
    torch = __import__("pytest").importorskip("torch")
    for sh in (W.Shape(12, 2, 1500, 30, 3, near_pole=0.02), W.Shape(5, 1, 257, 7, 4, igp_overflow=2)):
        a = W.make_inputs(sh, 23)
        b = W.make_inputs_device(sh, 23, device="cpu")
        for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul",
                  "inv_igp_index", "indinv", "wx_array"):
            np.testing.assert_array_equal(getattr(a, k), b[k].numpy(), err_msg=k)

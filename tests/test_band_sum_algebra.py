"""The algebra behind the band-sum GEMM paths, checked on the CPU in numpy
FP64 against the oracle: with one wx row for every band,

    achtemp[iw]     = sum_{r,ig} M_iw[r][ig] G[r][ig],  G = sum_{n1>=nv} c[n1][r] aqsn[n1][ig]
    acht_n1_loc[n1] = sum_r c[n1][r] H[n1][r],         H = sum_ig aqsn[n1][ig] M_2[r][ig]

with M_iw = wtilde I_eps conj(wdiff) / |wdiff|^2, wdiff = wx_iw - wtilde and
c = 0.5 vcoul[igp] conj(aqsm[n1][igp]) (igp clamped).  The unoccupied-band
part of the reference's sums equals these products; the occupied bands go
through the branchy solver and are left out (nvband = 0 here)."""
import numpy as np
import pytest

from gppsigma import workload as W


def band_sum(inp):
    s = inp.shape
    igp = np.minimum(inp.inv_igp_index, s.ncouls - 1)
    c = 0.5 * inp.vcoul[igp][None, :] * np.conj(inp.aqsmtemp[:, igp])  # [nb][ng]
    G = c[s.nvband:].T @ inp.aqsntemp[s.nvband:]                      # [ng][nc]
    wt, ie = inp.wtilde_array, inp.I_eps_array
    ach = np.zeros(s.nw, np.complex128)
    M2 = None
    for iw in range(s.nw):
        wdiff = inp.wx_array[0, iw] - wt
        M = wt * ie * np.conj(wdiff) / np.abs(wdiff) ** 2
        ach[iw] = np.sum(M * G)
        if iw == 2:
            M2 = M
    n1 = None
    if M2 is not None:
        H = inp.aqsntemp[s.nvband:] @ M2.T                             # [nb'][ng]
        n1 = np.zeros(s.number_bands, np.complex128)
        n1[s.nvband:] = np.sum(c[s.nvband:] * H, axis=1)
    return ach, n1


@pytest.mark.parametrize("shape", [W.Shape(12, 0, 300, 9, 3), W.Shape(7, 0, 129, 5, 4, igp_overflow=2),
                                   W.Shape(9, 0, 64, 3, 1)])
def test_band_sum_factorisation_matches_the_oracle(shape):
    import oracle_py
    inp = W.make_inputs(shape, 3)
    inp.wx_array = inp.wx_array[:1].copy()
    want = oracle_py.run(inp, "complex_seq")
    ach, n1 = band_sum(inp)
    scale = np.max(np.abs(want["achtemp"]))
    assert np.max(np.abs(ach - want["achtemp"])) <= 1e-12 * scale
    if n1 is not None:
        s1 = np.max(np.abs(want["acht_n1_loc"]))
        assert np.max(np.abs(n1 - want["acht_n1_loc"])) <= 1e-12 * s1

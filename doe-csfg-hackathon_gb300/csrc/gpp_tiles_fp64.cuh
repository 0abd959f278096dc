// gpp_tiles_fp64.cuh -- FP64 tile bodies of the GPP sigma kernels, shared by
// the one-state kernels (gpp_fp64.cu) and the persistent batched kernels.
//
// Algorithm (reference: noflagOCC_solver gppComplex_seq.cpp:131-150,
// flagOCC_solver :107-128, ssxt_scht_solver :16-63, driver :335-383).
// The unoccupied term is regrouped, exactly in real arithmetic, as
//
//   mygpvar1 aqsn (delw I_eps) = conj(aqsm[n1,igp]) * A * conj(wdiff) / |wdiff|^2
//   A = aqsn[n1,ig] * (wtilde[igp,ig] * I_eps[igp,ig]),  wdiff = wx - wtilde
//
// so conj(aqsm) leaves the ig sum (applied once per (n1,igp) in the block
// epilogue) and A is shared by all frequencies.  Per term the FP64 pipe then
// does 9 instructions: wdiff.re (DADD), |wdiff|^2 (DFMA), the reciprocal (3
// DFMA after a seed from the multi-function unit), A*conj(wdiff) (2 DFMA with
// the iw-independent products hoisted) and the accumulation (2 DFMA).
//
// Work decomposition: a tile is RG local G' rows x RN bands x NWC
// frequencies and all ncouls columns; the block's threads stride over ig, so
// every global load is a coalesced 16-byte double2 (ld.global.nc) and each
// loaded element is reused RN*NWC (rows) or RG*NWC (bands) times from
// registers.  Partial sums: per-thread registers -> warp shuffle tree ->
// shared-memory tree across warps -> one complex per tile and frequency in
// the workspace, summed over tiles in a fixed order by the reduction kernel.
#pragma once

#include "gpp_internal.cuh"

namespace gpp {

// One unoccupied-band tile in FP64: rows row_tile*RG.., bands
// band_begin + band_tile*RN.., frequencies iw_chunk*NWC..; `tile` is the
// tile's index inside this launch's block-partial segment.  red/S are
// shared-memory scratch of (THREADS/32)*K and K doubles, K = RN*RG*NWC*2.
template <int RN, int RG, int NWC, int THREADS>
__device__ __forceinline__ void noflag_fp64_tile(const Problem &p, const Partials &part,
                                                 int band_begin, int band_end, int row_tile,
                                                 int band_tile, int iw_chunk, long long tile,
                                                 double *red, double *S) {
    constexpr int K = RN * RG * NWC * 2;
    const int row0 = row_tile * RG;
    const int band0 = band_begin + band_tile * RN;
    const int iw0 = iw_chunk * NWC;
    const int nc = p.nc;

    const double2 *wrow[RG];
    const double2 *erow[RG];
#pragma unroll
    for (int g = 0; g < RG; ++g) {
        const int r = min(row0 + g, p.ng - 1);
        wrow[g] = p.wt + (size_t)r * nc;
        erow[g] = p.ieps + (size_t)r * nc;
    }
    const double2 *nrow[RN];
    double wx[RN][NWC];
#pragma unroll
    for (int n = 0; n < RN; ++n) {
        const int b = min(band0 + n, band_end - 1);
        nrow[n] = p.aqsn + (size_t)b * nc;
#pragma unroll
        for (int w = 0; w < NWC; ++w)
            wx[n][w] = __ldg(p.wx + (size_t)b * p.wx_stride + min(iw0 + w, p.nw - 1));
    }

    double2 acc[RN][RG][NWC];
#pragma unroll
    for (int n = 0; n < RN; ++n)
#pragma unroll
        for (int g = 0; g < RG; ++g)
#pragma unroll
            for (int w = 0; w < NWC; ++w) acc[n][g][w] = make_double2(0.0, 0.0);

    for (int ig = threadIdx.x; ig < nc; ig += THREADS) {
        double2 Q[RG];
        double wtr[RG], wti[RG], wti2[RG];
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            const double2 wt = __ldg(wrow[g] + ig);
            const double2 ie = __ldg(erow[g] + ig);
            Q[g] = cmul(wt, ie);
            wtr[g] = wt.x;
            wti[g] = wt.y;
            wti2[g] = wt.y * wt.y;
        }
#pragma unroll
        for (int n = 0; n < RN; ++n) {
            const double2 a = __ldg(nrow[n] + ig);
#pragma unroll
            for (int g = 0; g < RG; ++g) {
                const double2 A = cmul(a, Q[g]);
                const double ayw = A.y * wti[g];
                const double axw = A.x * wti[g];
#pragma unroll
                for (int w = 0; w < NWC; ++w) {
                    const double wr = wx[n][w] - wtr[g];   // Re(wdiff); Im(wdiff) = -wti
                    const double d = fma(wr, wr, wti2[g]); // |wdiff|^2
                    const double r = rcp_fp64(d);
                    const double tx = fma(A.x, wr, -ayw);  // A * conj(wdiff)
                    const double ty = fma(A.y, wr, axw);
                    acc[n][g][w].x = fma(r, tx, acc[n][g][w].x);
                    acc[n][g][w].y = fma(r, ty, acc[n][g][w].y);
                }
            }
        }
    }

    double v[K];
#pragma unroll
    for (int n = 0; n < RN; ++n)
#pragma unroll
        for (int g = 0; g < RG; ++g)
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                const int k = ((n * RG + g) * NWC + w) * 2;
                v[k] = acc[n][g][w].x;
                v[k + 1] = acc[n][g][w].y;
            }
    block_reduce<K, THREADS>(v, red, S);

    noflag_epilogue<RN, RG, NWC>(p, part, S, row0, band0, band_end, iw0, tile, row_tile);
}

// Epilogue of an occupied-band tile: S holds, per (row g, frequency w), the
// ig sums of aqsn*sch and aqsn*ssx as S[(g*NWC + w)*4 + {0,1 | 2,3}].  Weight
// by conj(aqsm[band,igp]) (the matngmatmgp factor) and by 0.5 vcoul[igp]
// (achtemp) or occ vcoul[igp] (asxtemp), gppComplex_seq.cpp:359-363,378-381;
// threads 0..NWC-1 write achtemp partials, NWC..2NWC-1 asxtemp partials and
// thread 64 the iw = 2 column of acht_n1_loc.
template <int RG, int NWC>
__device__ __forceinline__ void flag_epilogue(const Problem &p, const Partials &part,
                                              const double *S, int row0, int band, int iw0,
                                              long long tile, int row_tile) {
    const int nc = p.nc;
    const int t = threadIdx.x;
    // t < NWC: achtemp partial; NWC <= t < 2 NWC: asxtemp partial; t == 64: n1 column.
    const bool do_ach = t < NWC, do_asx = t >= NWC && t < 2 * NWC, do_n1 = part.n1 && t == 64;
    if (do_ach || do_asx || do_n1) {
        const int w = do_ach ? t : (do_asx ? t - NWC : 2 - iw0);
        if (w >= 0 && w < NWC && iw0 + w < p.nw) {
            double2 tot = make_double2(0.0, 0.0);
#pragma unroll
            for (int g = 0; g < RG; ++g) {
                const int row = row0 + g;
                if (row >= p.ng) continue;
                const int igp = resolve_igp(p, row, part.err);
                if (igp < 0) continue;
                const double2 m = __ldg(p.aqsm + (size_t)band * nc + igp);
                const int k = (g * NWC + w) * 4 + (do_asx ? 2 : 0);
                const double2 s =
                    cmul_rn(make_double2(m.x, -m.y), make_double2(S[k], S[k + 1]));
                const double v_igp = __ldg(p.vcoul + igp);
                const double2 t = do_asx ? cscale_rn(s, __dmul_rn(p.occ, v_igp))
                                         : cscale_rn(cscale_rn(s, 0.5), v_igp);
                tot = make_double2(__dadd_rn(tot.x, t.x), __dadd_rn(tot.y, t.y));
            }
            if (do_ach)
                part.ach[(long long)(iw0 + w) * part.ach_seg + part.ach_tile0 + tile] = tot;
            else if (do_asx)
                part.asx[(long long)(iw0 + w) * part.asx_seg + tile] = tot;
            else
                part.n1[(long long)band * part.n1_seg + row_tile] = tot;
        }
    }
}

// Per (row, column) factors of the occupied-band solver: wtilde^2 and
// Omega2 = wtilde^2 I_eps (gppComplex_seq.cpp:346-350).
__device__ __forceinline__ void flag_row_terms(double2 wt, double2 ie, double2 &wt2,
                                               double2 &om2) {
    wt2 = make_double2(__fma_rn(wt.x, wt.x, -__dmul_rn(wt.y, wt.y)),
                       __dmul_rn(__dmul_rn(2.0, wt.x), wt.y));
    om2 = cmul_rn(wt2, ie);
}

// ssxt_scht_solver (gppComplex_seq.cpp:16-63) for one (row, column,
// frequency): sch and ssx before the aqsn factor.  cwr = 1/wx^2 for branch A.
// Every rounding is explicit (the _rn helpers), so the one-band and the
// band-pair tiles produce the same bits.
template <int SEM>
__device__ __forceinline__ void flag_solve(double wx, double cwr, double2 wt, double2 wt2,
                                           double2 om2, double2 ie, double2 &sch_out,
                                           double2 &ssx_out) {
    const double2 wd = make_double2(__dsub_rn(wx, wt.x), -wt.y);
    const double wdr = abs2_rn(wd);
    const double rden = rcp_fp64(wdr);
    const double2 delw = cscale_rn(cmul_conj_b_rn(wt, wd), rden);
    const double delwr = abs2_rn(delw);
    double2 sch = make_double2(0.0, 0.0), ssx = make_double2(0.0, 0.0);
    if (wdr > kLimitTwo && delwr < kLimitOne) {
        sch = cmul_rn(delw, ie);
        ssx = cscale_rn(om2, cwr);
    } else if (delwr > kTo1) {
        const double2 cden =
            cscale_rn(cmul_rn(wt2, make_double2(__dadd_rn(0.5, delw.x), delw.y)), 4.0);
        const double r2 = rcp_fp64(abs2_rn(cden));
        ssx = cmul_rn(cmul_conj_b_rn(make_double2(-om2.x, -om2.y), cden), cscale_rn(delw, r2));
    }
    // |ssx| > sexcut |I_eps| compared on squares (sexcut^2 = 16 is exact).
    if (SEM == kSemComplexSeq && wx < 0.0 && abs2_rn(ssx) > __dmul_rn(16.0, abs2_rn(ie)))
        ssx = make_double2(0.0, 0.0);
    sch_out = sch;
    ssx_out = ssx;
}

// One occupied-band term, accumulated as aqsn*sch and aqsn*ssx (the
// conj(aqsm) factor of matngmatmgp is applied in the epilogue).
template <int SEM>
__device__ __forceinline__ void flag_term(double wx, double cwr, double2 wt, double2 wt2,
                                          double2 om2, double2 ie, double2 a, double2 &acc_s,
                                          double2 &acc_x) {
    double2 sch, ssx;
    flag_solve<SEM>(wx, cwr, wt, wt2, om2, ie, sch, ssx);
    acc_s = cmul_acc_rn(acc_s, a, sch);
    acc_x = cmul_acc_rn(acc_x, a, ssx);
}

// One occupied-band tile in FP64: rows row_tile*RG.., one band, frequencies
// iw_chunk*NWC..; `tile` indexes this launch's segment of block partials.
// red/S are shared scratch of (THREADS/32)*K and K doubles, K = RG*NWC*4.
template <int RG, int NWC, int THREADS, int SEM>
__device__ __forceinline__ void flag_fp64_tile(const Problem &p, const Partials &part,
                                               int row_tile, int band, int iw_chunk,
                                               long long tile, double *red, double *S) {
    constexpr int K = RG * NWC * 4;
    const int row0 = row_tile * RG;
    const int iw0 = iw_chunk * NWC;
    const int nc = p.nc;

    const double2 *wrow[RG];
    const double2 *erow[RG];
#pragma unroll
    for (int g = 0; g < RG; ++g) {
        const int r = min(row0 + g, p.ng - 1);
        wrow[g] = p.wt + (size_t)r * nc;
        erow[g] = p.ieps + (size_t)r * nc;
    }
    const double2 *nrow = p.aqsn + (size_t)band * nc;
    double wx[NWC], cwr[NWC];
#pragma unroll
    for (int w = 0; w < NWC; ++w) {
        wx[w] = __ldg(p.wx + (size_t)band * p.wx_stride + min(iw0 + w, p.nw - 1));
        const double c = wx[w] * wx[w];
        cwr[w] = c / (c * c);  // wx^2 / pow(wx^2, 2), once per (band, iw)
    }

    double2 acc_s[RG][NWC], acc_x[RG][NWC];
#pragma unroll
    for (int g = 0; g < RG; ++g)
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            acc_s[g][w] = make_double2(0.0, 0.0);
            acc_x[g][w] = make_double2(0.0, 0.0);
        }

    for (int ig = threadIdx.x; ig < nc; ig += THREADS) {
        const double2 a = __ldg(nrow + ig);
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            const double2 wt = __ldg(wrow[g] + ig);
            const double2 ie = __ldg(erow[g] + ig);
            double2 wt2, om2;
            flag_row_terms(wt, ie, wt2, om2);
#pragma unroll
            for (int w = 0; w < NWC; ++w)
                flag_term<SEM>(wx[w], cwr[w], wt, wt2, om2, ie, a, acc_s[g][w], acc_x[g][w]);
        }
    }

    double v[K];
#pragma unroll
    for (int g = 0; g < RG; ++g)
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            const int k = (g * NWC + w) * 4;
            v[k] = acc_s[g][w].x;
            v[k + 1] = acc_s[g][w].y;
            v[k + 2] = acc_x[g][w].x;
            v[k + 3] = acc_x[g][w].y;
        }
    block_reduce<K, THREADS>(v, red, S);
    flag_epilogue<RG, NWC>(p, part, S, row0, band, iw0, tile, row_tile);
}

// Occupied bands with band-independent frequencies (wx_stride == 0): the
// solver's sch / ssx depend on (row, column, frequency) only, so one tile
// evaluates them once for NB bands [band0, band0 + NB) and accumulates
// aqsn * sch, aqsn * ssx per band.  Per band the operations, their order and
// the reduction tree are those of flag_fp64_tile: the same bits, with 1/NB
// of the solver work.  Bands past nv (a ragged last group) are computed on a
// clamped band and not written.
template <int RG, int NWC, int NB, int THREADS, int SEM>
__device__ __forceinline__ void flag_fp64_multi_tile(const Problem &p, const Partials &part,
                                                     int row_tile, int band0, int iw_chunk,
                                                     int row_tiles, double *red, double *S) {
    constexpr int KB = RG * NWC * 4, K = NB * KB;
    const int row0 = row_tile * RG;
    const int iw0 = iw_chunk * NWC;
    const int nc = p.nc;

    const double2 *wrow[RG];
    const double2 *erow[RG];
#pragma unroll
    for (int g = 0; g < RG; ++g) {
        const int r = min(row0 + g, p.ng - 1);
        wrow[g] = p.wt + (size_t)r * nc;
        erow[g] = p.ieps + (size_t)r * nc;
    }
    const double2 *nrow[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) nrow[b] = p.aqsn + (size_t)min(band0 + b, p.nv - 1) * nc;
    double wx[NWC], cwr[NWC];
#pragma unroll
    for (int w = 0; w < NWC; ++w) {
        wx[w] = __ldg(p.wx + min(iw0 + w, p.nw - 1));  // the same for every band
        const double c = wx[w] * wx[w];
        cwr[w] = c / (c * c);
    }

    double2 acc_s[NB][RG][NWC], acc_x[NB][RG][NWC];
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int g = 0; g < RG; ++g)
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                acc_s[b][g][w] = make_double2(0.0, 0.0);
                acc_x[b][g][w] = make_double2(0.0, 0.0);
            }

    for (int ig = threadIdx.x; ig < nc; ig += THREADS) {
        double2 a[NB];
#pragma unroll
        for (int b = 0; b < NB; ++b) a[b] = __ldg(nrow[b] + ig);
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            const double2 wt = __ldg(wrow[g] + ig);
            const double2 ie = __ldg(erow[g] + ig);
            double2 wt2, om2;
            flag_row_terms(wt, ie, wt2, om2);
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                double2 sch, ssx;
                flag_solve<SEM>(wx[w], cwr[w], wt, wt2, om2, ie, sch, ssx);
#pragma unroll
                for (int b = 0; b < NB; ++b) {
                    acc_s[b][g][w] = cmul_acc_rn(acc_s[b][g][w], a[b], sch);
                    acc_x[b][g][w] = cmul_acc_rn(acc_x[b][g][w], a[b], ssx);
                }
            }
        }
    }

    double v[K];
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int g = 0; g < RG; ++g)
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                const int k = b * KB + (g * NWC + w) * 4;
                v[k] = acc_s[b][g][w].x;
                v[k + 1] = acc_s[b][g][w].y;
                v[k + 2] = acc_x[b][g][w].x;
                v[k + 3] = acc_x[b][g][w].y;
            }
    block_reduce<K, THREADS>(v, red, S);
#pragma unroll
    for (int b = 0; b < NB; ++b)
        if (band0 + b < p.nv)
            flag_epilogue<RG, NWC>(p, part, S + b * KB, row0, band0 + b, iw0,
                                   (long long)(band0 + b) * row_tiles + row_tile, row_tile);
}

}  // namespace gpp

// gpp_tiles_mixed.cuh -- the mixed-precision unoccupied-band tile of the GPP
// sigma reduction (float-float bulk, FP64 near the plasmon pole), shared by
// the one-state kernel (gpp_mixed.cu) and the persistent batched kernels.
#pragma once

#include <cstring>

#include "gpp_df.cuh"
#include "gpp_df2.cuh"
#include "gpp_internal.cuh"
#include "gpp_tiles_fp64.cuh"

namespace gpp {

// Split planes written by the prep kernels.  G' rows are stored in pairs
// (rows 2j and 2j+1; the second repeats row ng-1 when ng is odd) as four
// float4 planes per pair, so that one 16-byte load yields both rows' values
// as two aligned register pairs, the operands of the packed f32x2
// instructions:
//   rows[j][0][ig] = (wt.re hi of row 2j, hi of row 2j+1, lo of 2j, lo of 2j+1)
//   rows[j][1][ig] = the same for wt.im
//   rows[j][2][ig], rows[j][3][ig] = the same for Q.re, Q.im (Q = wt*I_eps, FP64)
// masks[j][k] has a bit for every value bucket (below) that Re(wtilde) hi of
// rows 2j, 2j+1 takes in columns 64k .. 64k+63, written by the row split.
// A warp skips the per-term pole test for a chunk when none of the chunk's
// buckets can hold a wtilde within the pole distance of its wx values.
struct SplitPlanes {
    float4 *rows;                 // [ceil(ng/2)][4][nc]
    float4 *band;                 // [nb][nc]: aqsn.re hi, lo, .im hi, lo
    float2 *wx;                   // [nb][nw]: wx hi, lo
    unsigned long long *masks;    // [ceil(ng/2)][ceil(nc/64)], zeroed before the split
};
constexpr int kMaskCols = 64;
// Monotonic map of floats onto unsigned integers (integer order = float
// order).
__host__ __device__ __forceinline__ unsigned float_key(float f) {
    unsigned u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
// Value bucket: the top 11 bits of the key (sign, exponent, two mantissa
// bits, in value order), hashed onto one of 64 mask bits.  Shared bits only
// cost a needless test, never a missed one.
__host__ __device__ __forceinline__ unsigned bucket_code(float f) { return float_key(f) >> 21; }
__host__ __device__ __forceinline__ unsigned long long bucket_bit(unsigned code) {
    return 1ull << ((code ^ (code >> 6)) & 63);
}
// Mask bits of every bucket a wtilde within the FP64 pole distance of x
// (|wdiff|^2 < 1e-6 x^2, so |x - Re(wtilde)| < 1e-3 |x|) can fall into, with
// a margin far above the float rounding of both sides; all bits for NaN.
__host__ __device__ __forceinline__ unsigned long long pole_buckets(float x) {
    const float rad = 1.01e-3f * fabsf(x) + 1e-30f;
    const float lo = x - rad, hi = x + rad;
    if (!(lo <= hi)) return ~0ull;
    const unsigned c0 = bucket_code(lo), c1 = bucket_code(hi);
    if (c1 - c0 >= 64) return ~0ull;
    unsigned long long m = 0;
    for (unsigned c = c0; c <= c1; ++c) m |= bucket_bit(c);
    return m;
}

// One row of a row pair's plane value: (hi, lo) of row 2j + g.
__device__ __forceinline__ df pair_lane(const float4 &v, int g) {
    return g == 0 ? df{v.x, v.z} : df{v.y, v.w};
}

// The full term in FP64 from the original inputs, for |wdiff| < 1e-3 |wx|.
static __device__ __noinline__ void pole_term_fp64(const Problem &p, int row, int band, int ig, int iw,
                                            df &re, df &im) {
    const double2 wt = __ldg(p.wt + (size_t)row * p.nc + ig);
    const double2 ie = __ldg(p.ieps + (size_t)row * p.nc + ig);
    const double2 a = __ldg(p.aqsn + (size_t)band * p.nc + ig);
    const double wx = __ldg(p.wx + (size_t)band * p.wx_stride + iw);
    const double2 A = cmul(a, cmul(wt, ie));
    const double wr = wx - wt.x;
    const double r = 1.0 / (wr * wr + wt.y * wt.y);
    const double tx = (A.x * wr - A.y * wt.y) * r;
    const double ty = (A.y * wr + A.x * wt.y) * r;
    re = split(tx);
    im = split(ty);
}

// ---------------------------------------------------------------------------
// Shared-memory pipeline primitives: 1-D bulk TMA copies (cp.async.bulk)
// completing on an mbarrier with a transaction count.
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void mbar_inval(unsigned long long *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait for phase `parity` of `bar`.  Gives up (returns false) after
// `limit` polls, or as soon as another thread of the block has raised
// *abort, so a block never spins without end.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity,
                                          volatile int *abort, int limit = kWaitLimit) {
    for (int it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63) == 63 && *abort) return false;
    }
    *abort = 1;
    return false;
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes,
                                              unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// The lanes of a term pair that lie near the pole (d.h < thr), recomputed in
// FP64 from the inputs.  Out of line and returning whole pairs by value, so
// the rare per-lane update does not split the pairs' registers in the hot
// loop.
struct TermPair {
    df2 re, im;
};
static __device__ __noinline__ TermPair pole_pair(const Problem &p, df2 d, float thr, int row0,
                                                  int band, int ig, int iw, TermPair t) {
    for (int g = 0; g < 2; ++g) {
        if (!((g == 0 ? d.h.x : d.h.y) >= thr)) {
            df x, y;
            pole_term_fp64(p, min(row0 + g, p.ng - 1), band, ig, iw, x, y);
            df2_set_lane(t.re, g, x);
            df2_set_lane(t.im, g, y);
        }
    }
    return t;
}

// The df arithmetic of one ig column for one warp: RNW bands x the tile's
// two rows x NWC frequencies of aqsn * Q * conj(wdiff) / |wdiff|^2 added into
// acc.  Every value is a df2 whose lanes are rows row0 and row0 + 1, so one
// packed f32x2 instruction advances both rows' terms; the row-pair planes
// load straight into lane pairs and band values broadcast to both lanes.
// Re(wdiff) is renormalised after its cancelling subtraction and the
// reciprocal carries a second-order correction, folded into the two
// products by 1/|wdiff|^2 (df2_mul_rcp): both keep the per-term error near
// 2^-44 relative and free of a sign preference (an unnormalised wdiff or a
// first-order reciprocal biases every term the same way, and sums of 1e10
// terms turn a 1e-15 bias into 1e-10; tests/test_error_budget.py measures
// each step).  With CHECK, terms within 1e-3 |wx| of the pole are
// recomputed in FP64 from the inputs; tiles call the CHECK = false form only
// when no wtilde can come that near any of the warp's wx values.
template <int RNW, int NWC, int KC, bool CHECK>
__device__ __forceinline__ void mixed_column(const Problem &p, const float4 *st,
                                             const float4 *sb, int il, int ig, int row0,
                                             int bandw, int band_end, int iw0,
                                             const df (&wx)[RNW][NWC],
                                             const float (&pole_thr)[RNW][NWC],
                                             df2 (&acc)[RNW][NWC][2]) {
    const float4 vr = st[il], vi = st[KC + il], vqr = st[2 * KC + il], vqi = st[3 * KC + il];
    const df2 wtr = {f2(vr.x, vr.y), f2(vr.z, vr.w)};
    const df2 wti = {f2(vi.x, vi.y), f2(vi.z, vi.w)};
    const df2 qr = {f2(vqr.x, vqr.y), f2(vqr.z, vqr.w)};
    const df2 qi = {f2(vqi.x, vqi.y), f2(vqi.z, vqi.w)};
    const df2 wti2 = df2_mul(wti, wti);
#pragma unroll
    for (int n = 0; n < RNW; ++n) {
        const float4 av = sb[n * KC + il];
        const df2 ar = df2_bcast(df{av.x, av.y}), ai = df2_bcast(df{av.z, av.w});
        // A = aqsn * Q (frequency independent)
        const df2 Ar = df2_sub(df2_mul(ar, qr), df2_mul(ai, qi));
        const df2 Ai = df2_add(df2_mul(ar, qi), df2_mul(ai, qr));
        const df2 Ai_wti = df2_mul(Ai, wti);
        const df2 Ar_wti = df2_mul(Ar, wti);
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            const df2 wr = df2_norm(df2_sub(df2_bcast(wx[n][w]), wtr));  // Re(wdiff)
            const df2 d = df2_add(df2_sqr(wr), wti2);                     // |wdiff|^2
            float2 r0, rc;                              // 1/d = r0 (1 + rc)
            df2_rcp_parts(d, r0, rc);
            // A conj(wdiff) / |wdiff|^2, conj(wdiff) = (wr, wti)
            df2 tre = df2_mul_rcp(df2_sub(df2_mul(Ar, wr), Ai_wti), r0, rc);
            df2 tim = df2_mul_rcp(df2_add(df2_mul(Ai, wr), Ar_wti), r0, rc);
            if (CHECK) {
                const float thr = pole_thr[n][w];
                if (!(d.h.x >= thr) || !(d.h.y >= thr)) {
                    const TermPair t = pole_pair(p, d, thr, row0, min(bandw + n, band_end - 1),
                                                 ig, min(iw0 + w, p.nw - 1), TermPair{tre, tim});
                    tre = t.re;
                    tim = t.im;
                }
            }
            acc[n][w][0] = df2_add(acc[n][w][0], tre);
            acc[n][w][1] = df2_add(acc[n][w][1], tim);
        }
    }
}

enum : int { kSyncBlock = 0, kSyncRing = 1 };

// Unoccupied bands, mixed precision.  A block owns RG local G' rows and
// NWARP * RNW bands; warp w owns bands band0 + w*RNW .. +RNW-1.  The ig range
// is processed in chunks of KC columns through an NSTAGE-deep shared-memory
// ring: thread 0 streams each chunk's row-pair planes (wt.re, wt.im, Q.re,
// Q.im: 4 x KC x 16 B) and band planes (aqsn: NWARP*RNW x KC x 16 B) into a
// stage with 1-D bulk TMA copies that complete on the stage's "full"
// mbarrier; each warp reads the rows (one copy serves all warps) and its own
// bands, lanes on consecutive ig (conflict-free 16-byte LDS).  Two ways to recycle a stage:
//  * kSyncBlock: one __syncthreads per chunk; the refill of the stage read in
//    the previous chunk is issued right after it, NSTAGE-1 chunks ahead;
//  * kSyncRing: each warp arrives on the stage's "empty" mbarrier, and the
//    producer refills a stage one chunk behind the consumers, so warps run
//    decoupled without block-wide barriers.
// Per-lane df sums are reduced across the warp with a fixed shuffle tree in
// df arithmetic, converted to FP64 once, and combined by the common epilogue.
// Every wait is bounded (kWaitLimit polls, or an abort raised by another
// thread of the block); a block that gives up records kErrPipelineTimeout.
// One unoccupied-band tile in mixed precision: rows row_tile*RG.., bands
// band_begin + band_tile*BN.., frequencies iw_chunk*NWC..; `tile` indexes the
// launch's segment of block partials.  `reinit` must be set when the block
// ran an earlier tile with the same barriers (persistent kernels).  Returns
// false if the tile was abandoned after a bounded wait ran out.
template <int RNW, int RG, int NWC, int NWARP, int KC, int NSTAGE, int SYNC>
__device__ __forceinline__ bool mixed_tile(const Problem &p, const Partials &part,
                                           const SplitPlanes &s, int band_begin, int band_end,
                                           int row_tile, int band_tile, int iw_chunk,
                                           long long tile, bool reinit) {
    constexpr int BN = NWARP * RNW;            // bands per block
    constexpr int K = BN * RG * NWC * 2;       // doubles in the block result
    constexpr int STAGE = (2 * RG + BN) * KC;  // float4 per stage
    static_assert(KC % 32 == 0, "chunk must be a multiple of the warp width");
    static_assert(NSTAGE >= 2, "need at least two stages");
    static_assert(RG == 2, "tiles cover one row pair of the split planes");
    // Two columns per loop trip give the scheduler independent work (0.8%
    // faster with 3 frequencies); the 8-frequency tile, already at its
    // register cap, runs one.
    constexpr int kColUnroll = NWC <= 4 ? 2 : 1;
    extern __shared__ __align__(128) float4 stage_mem[];
    __shared__ unsigned long long full_bar[NSTAGE], empty_bar[NSTAGE];
    __shared__ int abort_flag;
    __shared__ double S[K];

    const int row0 = row_tile * RG;
    const int band0 = band_begin + band_tile * BN;
    const int iw0 = iw_chunk * NWC;
    const int nc = p.nc;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bandw = band0 + warp * RNW;
    const int nchunks = (nc + KC - 1) / KC;
    volatile int *abort = &abort_flag;

    // Producer: copy chunk c into stage c % NSTAGE.
    auto issue = [&](int c) {
        const int k0 = c * KC;
        const int cnt = min(KC, nc - k0);
        const unsigned bytes = (unsigned)cnt * 16u;
        float4 *st = stage_mem + (c % NSTAGE) * STAGE;
        unsigned long long *bar = &full_bar[c % NSTAGE];
        mbar_expect_tx(bar, bytes * (2 * RG + BN));
        // The row pair's four planes (wt.re, wt.im, Q.re, Q.im).
        const size_t r = (size_t)row_tile * 4 * nc + k0;
#pragma unroll
        for (int k = 0; k < 4; ++k) bulk_copy_g2s(st + k * KC, s.rows + r + (size_t)k * nc, bytes, bar);
#pragma unroll
        for (int n = 0; n < BN; ++n) {
            const size_t b = (size_t)min(band0 + n, band_end - 1) * nc + k0;
            bulk_copy_g2s(st + (2 * RG + n) * KC, s.band + b, bytes, bar);
        }
    };

    __syncthreads();  // the previous tile of this block is done with the barriers
    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int i = 0; i < NSTAGE; ++i) {
            if (reinit) {
                mbar_inval(&full_bar[i]);
                mbar_inval(&empty_bar[i]);
            }
            mbar_init(&full_bar[i], 1);
            mbar_init(&empty_bar[i], NWARP);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int issued = 0;  // chunks issued so far (thread 0 only)
    if (threadIdx.x == 0)
        for (; issued < NSTAGE - 1 && issued < nchunks; ++issued) issue(issued);

    df wx[RNW][NWC];
    float pole_thr[RNW][NWC];
    unsigned long long pole_mask = 0;  // value buckets of a possible pole term
    const unsigned long long *mask_row =
        s.masks + (size_t)row_tile * ((nc + kMaskCols - 1) / kMaskCols);
#pragma unroll
    for (int n = 0; n < RNW; ++n) {
        const int b = min(bandw + n, band_end - 1);
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            const float2 x = s.wx[(size_t)b * p.nw + min(iw0 + w, p.nw - 1)];
            wx[n][w] = {x.x, x.y};
            pole_thr[n][w] = 1e-6f * x.x * x.x;  // |wdiff|^2 < (1e-3 |wx|)^2
            pole_mask |= pole_buckets(x.x);
        }
    }
    df2 acc[RNW][NWC][2];  // lanes: the two rows
#pragma unroll
    for (int n = 0; n < RNW; ++n)
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            acc[n][w][0] = {f2(0.f, 0.f), f2(0.f, 0.f)};
            acc[n][w][1] = {f2(0.f, 0.f), f2(0.f, 0.f)};
        }

    int c_stop = nchunks;  // first chunk thread 0 did not consume
    for (int c = 0; c < nchunks; ++c) {
        // Refill the stage that chunk c - 1 used with chunk c + NSTAGE - 1.
        if (threadIdx.x == 0 && issued < nchunks && !*abort) {
            if (SYNC == kSyncBlock || issued < NSTAGE) {
                if (issued >= NSTAGE) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(issued++);
            } else {
                const int sp = issued % NSTAGE;
                const unsigned par = (unsigned)((issued / NSTAGE - 1) & 1);
                if (mbar_wait(&empty_bar[sp], par, abort)) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue(issued++);
                }
            }
        }
        if (SYNC == kSyncRing && warp == 0) __syncwarp();  // warp 0 waits for its producer lane
        // Value buckets of this chunk's wtilde (read before the wait).
        unsigned long long chunk_mask = 0;
        for (int k = (c * KC) / kMaskCols; k <= (min(c * KC + KC, nc) - 1) / kMaskCols; ++k)
            chunk_mask |= __ldg(mask_row + k);
        const int sidx = c % NSTAGE;
        const bool ok = mbar_wait(&full_bar[sidx], (unsigned)((c / NSTAGE) & 1), abort);
        if (ok) {
            const float4 *st = stage_mem + sidx * STAGE;      // row planes
            const float4 *sb = st + (2 * RG + warp * RNW) * KC;  // this warp's bands
            const int k0 = c * KC;
            const int cnt = min(KC, nc - k0);
            if (chunk_mask & pole_mask) {
#pragma unroll kColUnroll
                for (int il = lane; il < cnt; il += 32)
                    mixed_column<RNW, NWC, KC, true>(p, st, sb, il, k0 + il, row0, bandw,
                                                     band_end, iw0, wx, pole_thr, acc);
            } else {
#pragma unroll kColUnroll
                for (int il = lane; il < cnt; il += 32)
                    mixed_column<RNW, NWC, KC, false>(p, st, sb, il, k0 + il, row0, bandw,
                                                      band_end, iw0, wx, pole_thr, acc);
            }
        }
        if (SYNC == kSyncBlock) {
            __syncthreads();  // every warp is done with stage sidx
            if (*abort) {
                c_stop = c;
                break;
            }
        } else {
            if (!ok) {
                c_stop = c;
                break;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty_bar[sidx]);
        }
    }

    if (__syncthreads_or(*abort)) {
        if (threadIdx.x == 0) {
            atomicOr(part.err, kErrPipelineTimeout);
            // Let the copies still in flight land before the block retires.
            for (int j = c_stop; j < issued; ++j) {
                int spin = 0;
                while (!mbar_try_wait(&full_bar[j % NSTAGE], (unsigned)((j / NSTAGE) & 1)) &&
                       ++spin < kWaitLimit) {
                }
            }
        }
        return false;
    }

    // Warp tree in df arithmetic (fixed order), then one FP64 value per
    // (band, row, frequency) and component into shared memory.
#pragma unroll
    for (int n = 0; n < RNW; ++n)
#pragma unroll
        for (int g = 0; g < RG; ++g)
#pragma unroll
            for (int w = 0; w < NWC; ++w)
#pragma unroll
                for (int ri = 0; ri < 2; ++ri) {
                    df v;
                    v = df2_lane(acc[n][w][ri], g);
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) {
                        const df o = {__shfl_down_sync(0xffffffffu, v.h, off),
                                      __shfl_down_sync(0xffffffffu, v.l, off)};
                        v = df_add(v, o);
                    }
                    if (lane == 0)
                        S[(((warp * RNW + n) * RG + g) * NWC + w) * 2 + ri] = to_double(v);
                }
    __syncthreads();
    noflag_epilogue<BN, RG, NWC>(p, part, S, row0, band0, band_end, iw0, tile, row_tile);
    return true;
}

// ---------------------------------------------------------------------------
// Occupied bands (ssxt_scht_solver, gppComplex_seq.cpp:16-63) in float-float.

// a > t for a df value with |a.l| <= ~2^-22 |a.h| and a normalised df
// threshold t: decided on the high parts unless they are within 1e-5 of each
// other, then on the exact df difference.  Avoids branch flips at rounding
// level against the FP64 reference.
__device__ __forceinline__ bool df_gt(df a, df t) {
    const float d = fsub(a.h, t.h);
    if (fabsf(d) > 1e-5f * fabsf(t.h)) return d > 0.f;
    const df e = df_norm(df_sub(a, t));
    return e.h > 0.f || (e.h == 0.f && e.l > 0.f);
}
// The solver's thresholds (limittwo, limitone, to1) as float-float values,
// rounded at compile time: converted on the device, the compiler may
// recompute them (FP64 conversions) inside the term loop.
constexpr float kLim2H = (float)kLimitTwo, kLim2L = (float)(kLimitTwo - (double)kLim2H);
constexpr float kLim1H = (float)kLimitOne, kLim1L = (float)(kLimitOne - (double)kLim1H);
constexpr float kTo1H = (float)kTo1, kTo1L = (float)(kTo1 - (double)kTo1H);
__device__ __forceinline__ df df_abs2(df re, df im) { return df_add(df_sqr(re), df_sqr(im)); }
// (a.re + i a.im) * (b.re + i b.im) in df.
__device__ __forceinline__ void df_cmul(df ar, df ai, df br, df bi, df &cr, df &ci) {
    cr = df_sub(df_mul(ar, br), df_mul(ai, bi));
    ci = df_add(df_mul(ar, bi), df_mul(ai, br));
}
__device__ __forceinline__ df df_scale(df a, float k) { return {fmul(a.h, k), fmul(a.l, k)}; }

// An occupied-band term near the pole, in FP64 from the original inputs,
// split to float-float: aqsn*sch (sr, si) and aqsn*ssx (xr, xi).  Out of line:
// inlined, its FP64 code took registers from the float-float term loop.
struct FlagPole {
    df sr, si, xr, xi;
};
template <int SEM>
static __device__ __noinline__ FlagPole flag_pole(const Problem &p, int row, int band, int ig,
                                                  double wx, double cwr) {
    const size_t nc = (size_t)p.nc;
    const double2 wt = __ldg(p.wt + (size_t)row * nc + ig);
    const double2 ie = __ldg(p.ieps + (size_t)row * nc + ig);
    const double2 a = __ldg(p.aqsn + (size_t)band * nc + ig);
    double2 wt2, om2;
    flag_row_terms(wt, ie, wt2, om2);
    double2 s64 = make_double2(0.0, 0.0), x64 = make_double2(0.0, 0.0);
    flag_term<SEM>(wx, cwr, wt, wt2, om2, ie, a, s64, x64);
    return {split(s64.x), split(s64.y), split(x64.x), split(x64.y)};
}

// One occupied-band tile in mixed precision: rows row_tile*RG.., one band,
// frequencies iw_chunk*NWC..; reads the float-float split planes (bands
// [0, nvband) must have been split too).  Per term, on df values:
//   wdiff, |wdiff|^2, rden = 1/|wdiff|^2, delwr = |delw|^2 = |wtilde|^2 rden;
//   branch A (|wdiff|^2 > limittwo, delwr < limitone):
//     aqsn*sch = A conj(wdiff) rden with A = aqsn Q,  aqsn*ssx = (aqsn Omega2) / wx^2
//     (the 1/wx^2 factor is applied to the ig sum, in FP64);
//   branch B (delwr > to1): sch = 0, ssx = -Omega2 conj(cden) delw / |cden|^2,
//     cden = 4 wtilde^2 (0.5 + delw);
//   cutoff |ssx|^2 |wtilde|^2 > 16 |Q|^2 (= |ssx| > 4 |I_eps|) when wx < 0
//   under COMPLEX_SEQ semantics.
// Terms within 1e-3 |wx| of the pole are computed in FP64 from the inputs.
template <int RG, int NWC, int THREADS, int SEM>
__device__ __forceinline__ void flag_mixed_tile(const Problem &p, const Partials &part,
                                                const SplitPlanes &s, int row_tile, int band,
                                                int iw_chunk, long long tile, double *red,
                                                double *S) {
    static_assert(RG == 2, "tiles cover one row pair of the split planes");
    constexpr int K = RG * NWC * 4;
    const int row0 = row_tile * RG;
    const int iw0 = iw_chunk * NWC;
    const int nc = p.nc;
    const df kLim2 = {kLim2H, kLim2L}, kLim1 = {kLim1H, kLim1L}, kT1 = {kTo1H, kTo1L};

    const float4 *rp = s.rows + (size_t)row_tile * 4 * nc;  // this row pair's planes
    const float4 *bp = s.band + (size_t)band * nc;
    df wx[NWC], cwr2[NWC];
    double wx64[NWC], cwr[NWC];
    float thr[NWC];
    bool cut_on[NWC];  // the ssx cutoff applies (COMPLEX_SEQ, wx < 0); no FP64 test per term
#pragma unroll
    for (int w = 0; w < NWC; ++w) {
        wx64[w] = __ldg(p.wx + (size_t)band * p.wx_stride + min(iw0 + w, p.nw - 1));
        wx[w] = split(wx64[w]);
        const double c = wx64[w] * wx64[w];
        cwr[w] = c / (c * c);  // wx^2 / pow(wx^2, 2) (gppComplex_seq.cpp:38-41)
        cwr2[w] = split(cwr[w] * cwr[w]);
        thr[w] = 1e-6f * wx[w].h * wx[w].h;
        cut_on[w] = SEM == kSemComplexSeq && wx64[w] < 0.0;
    }
    // Accumulators: aqsn*sch, sum of aqsn*Omega2 over branch-A terms (times
    // 1/wx^2 later), aqsn*ssx of branch-B and pole terms.
    df as_r[RG][NWC], as_i[RG][NWC], xa_r[RG][NWC], xa_i[RG][NWC], xb_r[RG][NWC], xb_i[RG][NWC];
#pragma unroll
    for (int g = 0; g < RG; ++g)
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            as_r[g][w] = as_i[g][w] = xa_r[g][w] = xa_i[g][w] = xb_r[g][w] = xb_i[g][w] =
                df{0.f, 0.f};
        }

    for (int ig = threadIdx.x; ig < nc; ig += THREADS) {
        const float4 av = __ldg(bp + ig);
        const df ar = {av.x, av.y}, ai = {av.z, av.w};
        const float4 pwr = __ldg(rp + ig), pwi = __ldg(rp + nc + ig);
        const float4 pqr = __ldg(rp + 2 * nc + ig), pqi = __ldg(rp + 3 * nc + ig);
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            const df wtr = pair_lane(pwr, g), wti = pair_lane(pwi, g);
            const df qr = pair_lane(pqr, g), qi = pair_lane(pqi, g);
            const df wti2 = df_sqr(wti);
            const df awt2 = df_add(df_sqr(wtr), wti2);                         // |wtilde|^2
            df w2r, w2i;                                                          // wtilde^2
            df_cmul(wtr, wti, wtr, wti, w2r, w2i);
            df omr, omi;                                                          // Omega2 = wtilde Q
            df_cmul(wtr, wti, qr, qi, omr, omi);
            const df cut_rhs = df_scale(df_abs2(qr, qi), 16.f);                  // 16 |Q|^2
            const df om_wt = df_mul(df_abs2(omr, omi), awt2);                   // |Omega2|^2 |wtilde|^2
            df Ar, Ai, Br, Bi;
            df_cmul(ar, ai, qr, qi, Ar, Ai);                                      // aqsn Q
            df_cmul(ar, ai, omr, omi, Br, Bi);                                    // aqsn Omega2
            const df Ai_wti = df_mul(Ai, wti), Ar_wti = df_mul(Ar, wti);
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                const df wr = df_norm(df_sub(wx[w], wtr));   // Re(wdiff); Im(wdiff) = -wti
                const df d = df_add(df_sqr(wr), wti2);       // |wdiff|^2
                if (d.h < thr[w]) {
                    // Near the pole: the whole term in FP64 from the inputs.
                    const FlagPole t = flag_pole<SEM>(p, min(row0 + g, p.ng - 1), band, ig,
                                                      wx64[w], cwr[w]);
                    as_r[g][w] = df_add(as_r[g][w], t.sr);
                    as_i[g][w] = df_add(as_i[g][w], t.si);
                    xb_r[g][w] = df_add(xb_r[g][w], t.xr);
                    xb_i[g][w] = df_add(xb_i[g][w], t.xi);
                    continue;
                }
                const df rden = df_rcp(d);
                const df delwr = df_mul(awt2, rden);
                if (df_gt(d, kLim2) && df_gt(kLim1, delwr)) {
                    // Branch A: aqsn*sch = A conj(wdiff) rden; aqsn*ssx = B / wx^2.
                    const df tre = df_mul(df_sub(df_mul(Ar, wr), Ai_wti), rden);
                    const df tim = df_mul(df_add(df_mul(Ai, wr), Ar_wti), rden);
                    as_r[g][w] = df_add(as_r[g][w], tre);
                    as_i[g][w] = df_add(as_i[g][w], tim);
                    const bool cut = cut_on[w] && df_gt(df_mul(om_wt, cwr2[w]), cut_rhs);
                    if (!cut) {
                        xa_r[g][w] = df_add(xa_r[g][w], Br);
                        xa_i[g][w] = df_add(xa_i[g][w], Bi);
                    }
                } else if (df_gt(delwr, kT1)) {
                    // Branch B.  delw = wtilde conj(wdiff) rden, conj(wdiff) = (wr, wti).
                    df dr, di;
                    df_cmul(wtr, wti, wr, wti, dr, di);
                    dr = df_mul(dr, rden);
                    di = df_mul(di, rden);
                    df cr, ci;                                   // cden = 4 wtilde^2 (0.5 + delw)
                    df_cmul(w2r, w2i, df_add(dr, df{0.5f, 0.f}), di, cr, ci);
                    cr = df_scale(cr, 4.f);
                    ci = df_scale(ci, 4.f);
                    const df r2 = df_rcp(df_norm(df_abs2(cr, ci)));
                    df tr, ti;                                   // -Omega2 conj(cden)
                    df_cmul(omr, omi, cr, df{-ci.h, -ci.l}, tr, ti);
                    df sr, si;                                   // ssx = -(...) (delw r2)
                    df_cmul(tr, ti, df_mul(dr, r2), df_mul(di, r2), sr, si);
                    sr = df{-sr.h, -sr.l};
                    si = df{-si.h, -si.l};
                    const bool cut =
                        cut_on[w] && df_gt(df_mul(df_abs2(sr, si), awt2), cut_rhs);
                    if (!cut) {
                        df pr, pi;
                        df_cmul(ar, ai, sr, si, pr, pi);
                        xb_r[g][w] = df_add(xb_r[g][w], pr);
                        xb_i[g][w] = df_add(xb_i[g][w], pi);
                    }
                }
            }
        }
    }

    double v[K];
#pragma unroll
    for (int g = 0; g < RG; ++g)
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            const int k = (g * NWC + w) * 4;
            v[k] = to_double(as_r[g][w]);
            v[k + 1] = to_double(as_i[g][w]);
            v[k + 2] = to_double(xa_r[g][w]) * cwr[w] + to_double(xb_r[g][w]);
            v[k + 3] = to_double(xa_i[g][w]) * cwr[w] + to_double(xb_i[g][w]);
        }
    block_reduce<K, THREADS>(v, red, S);
    flag_epilogue<RG, NWC>(p, part, S, row0, band, iw0, tile, row_tile);
}

}  // namespace gpp

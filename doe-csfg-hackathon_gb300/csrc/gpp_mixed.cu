// gpp_mixed.cu -- mixed-precision unoccupied-band kernel of the GPP sigma
// reduction for sm_103a.
//
// Why mixed precision pays on GB300: the FP64 pipe retires ~2 FMA/clk/SM
// against ~128 FP32 FMA/clk/SM, so an FP64 operation costs as much issue time
// as ~64 FP32 operations.  The bulk of every term therefore runs in
// float-float ("df") arithmetic: a value is an unevaluated sum hi + lo of two
// floats (~48 significant bits), combined with the error-free transformations
// TwoSum (Knuth) and FMA-based TwoProduct (Dekker; Ogita, Rump & Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).  Rounding
// errors of the main path are captured exactly; only second-order cross
// terms round in FP32, so each term carries ~2^-44 relative error, far below
// the 1e-8 target, while costing ~85 FP32 instructions instead of ~11 FP64
// ones (~700 FP32-equivalents).
//
// FP64 is kept where stability needs it:
//  * the input conversion: a prep pass computes Q = wtilde * I_eps in FP64 and
//    splits wtilde, Q, aqsn and wx into float hi/lo planes once per call
//    (memory-bound, ~1% of the kernel time), so no FP64 conversion sits in
//    the hot loop;
//  * near the plasmon pole, |wdiff| < 1e-3 |wx|, the whole term (wdiff, the
//    division, the products) is recomputed in FP64 from the original inputs;
//  * the cross-thread, cross-block and final sums (FP64 trees, fixed order).
//
// Work decomposition matches the FP64 kernel (RG rows x RN bands x NWC
// frequencies per block, threads striding over ig, 16-byte vector loads) with
// a grouped tile order so that GROUP row tiles stay resident in L2 while all
// band tiles stream past them.
#include "gpp_df.cuh"
#include "gpp_kernels.h"

namespace gpp {

namespace {

// Split planes written by the prep kernels (all float4 = 16 bytes).
struct SplitPlanes {
    float4 *rowW;  // [ng][nc]: wt.re hi, lo, wt.im hi, lo
    float4 *rowQ;  // [ng][nc]: (wt*I_eps).re hi, lo, .im hi, lo
    float4 *band;  // [nb][nc]: aqsn.re hi, lo, .im hi, lo
    float2 *wx;    // [nb][nw]: wx hi, lo
};

SplitPlanes planes(const Problem &p, void *ws) {
    char *w = static_cast<char *>(ws);
    SplitPlanes s;
    const size_t rows = (size_t)p.ng * p.nc, bands = (size_t)p.nb * p.nc;
    s.rowW = reinterpret_cast<float4 *>(w);
    s.rowQ = s.rowW + rows;
    s.band = s.rowQ + rows;
    s.wx = reinterpret_cast<float2 *>(s.band + bands);
    return s;
}

__global__ void __launch_bounds__(256) split_rows_kernel(Problem p, SplitPlanes s) {
    const size_t n = (size_t)p.ng * p.nc;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) {
        const double2 wt = __ldg(p.wt + i);
        const double2 ie = __ldg(p.ieps + i);
        const double2 q = cmul(wt, ie);
        const df wr = split(wt.x), wi = split(wt.y), qr = split(q.x), qi = split(q.y);
        s.rowW[i] = make_float4(wr.h, wr.l, wi.h, wi.l);
        s.rowQ[i] = make_float4(qr.h, qr.l, qi.h, qi.l);
    }
}

__global__ void __launch_bounds__(256) split_bands_kernel(Problem p, SplitPlanes s, int b0,
                                                          int b1) {
    const size_t n = (size_t)(b1 - b0) * p.nc;
    const size_t base = (size_t)b0 * p.nc;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) {
        const double2 a = __ldg(p.aqsn + base + i);
        const df ar = split(a.x), ai = split(a.y);
        s.band[base + i] = make_float4(ar.h, ar.l, ai.h, ai.l);
    }
    const int nwx = (b1 - b0) * p.nw;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < nwx; i += gridDim.x * 256) {
        const int b = b0 + i / p.nw, iw = i % p.nw;
        const df x = split(__ldg(p.wx + (size_t)b * p.wx_stride + iw));
        s.wx[(size_t)b * p.nw + iw] = make_float2(x.h, x.l);
    }
}

// The full term in FP64 from the original inputs, for |wdiff| < 1e-3 |wx|.
__device__ __noinline__ void pole_term_fp64(const Problem &p, int row, int band, int ig, int iw,
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
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait for phase `parity` of `bar`.  Gives up (returns false) after
// kWaitLimit polls, or as soon as another thread of the block has raised
// *abort, so a block never spins without end.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity,
                                          volatile int *abort) {
    for (int it = 0; it < kWaitLimit; ++it) {
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

// The df arithmetic of one ig column for one warp: RNW bands x RG rows x NWC
// frequencies of aqsn * Q * conj(wdiff) / |wdiff|^2 added into acc.  Terms
// within 1e-3 |wx| of the pole are recomputed in FP64 from the inputs.
template <int RNW, int RG, int NWC, int KC>
__device__ __forceinline__ void mixed_column(const Problem &p, const float4 *st,
                                             const float4 *sb, int il, int ig,
                                             int row0, int bandw, int band_end, int iw0,
                                             const df (&wx)[RNW][NWC],
                                             const float (&pole_thr)[RNW][NWC],
                                             df (&acc)[RNW][RG][NWC][2]) {
    df wtr[RG], wti[RG], wti2[RG], qr[RG], qi[RG];
#pragma unroll
    for (int g = 0; g < RG; ++g) {
        const float4 wv = st[g * KC + il];
        const float4 qv = st[(RG + g) * KC + il];
        wtr[g] = df{wv.x, wv.y};
        wti[g] = df{wv.z, wv.w};
        qr[g] = df{qv.x, qv.y};
        qi[g] = df{qv.z, qv.w};
        wti2[g] = df_sqr(wti[g]);
    }
#pragma unroll
    for (int n = 0; n < RNW; ++n) {
        const float4 av = sb[n * KC + il];
        const df ar = {av.x, av.y}, ai = {av.z, av.w};
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            // A = aqsn * Q (frequency independent)
            const df Ar = df_sub(df_mul(ar, qr[g]), df_mul(ai, qi[g]));
            const df Ai = df_add(df_mul(ar, qi[g]), df_mul(ai, qr[g]));
            const df Ai_wti = df_mul(Ai, wti[g]);
            const df Ar_wti = df_mul(Ar, wti[g]);
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                const df wr = df_norm(df_sub(wx[n][w], wtr[g]));  // Re(wdiff)
                const df d = df_add(df_sqr(wr), wti2[g]);         // |wdiff|^2
                df tre, tim;
                if (d.h >= pole_thr[n][w]) {
                    const df r = df_rcp(d);
                    // A * conj(wdiff) / |wdiff|^2, conj(wdiff) = (wr, wti)
                    tre = df_mul(df_sub(df_mul(Ar, wr), Ai_wti), r);
                    tim = df_mul(df_add(df_mul(Ai, wr), Ar_wti), r);
                } else {
                    pole_term_fp64(p, min(row0 + g, p.ng - 1), min(bandw + n, band_end - 1), ig,
                                   min(iw0 + w, p.nw - 1), tre, tim);
                }
                acc[n][g][w][0] = df_add(acc[n][g][w][0], tre);
                acc[n][g][w][1] = df_add(acc[n][g][w][1], tim);
            }
        }
    }
}

enum : int { kSyncBlock = 0, kSyncRing = 1 };

// Unoccupied bands, mixed precision.  A block owns RG local G' rows and
// NWARP * RNW bands; warp w owns bands band0 + w*RNW .. +RNW-1.  The ig range
// is processed in chunks of KC columns through an NSTAGE-deep shared-memory
// ring: thread 0 streams each chunk's row planes (wtilde, Q: RG x KC x 16 B
// each) and band planes (aqsn: NWARP*RNW x KC x 16 B) into a stage with 1-D
// bulk TMA copies that complete on the stage's "full" mbarrier; each warp
// reads the rows (one copy serves all warps) and its own bands, lanes on
// consecutive ig (conflict-free 16-byte LDS).  Two ways to recycle a stage:
//  * kSyncBlock: one __syncthreads per chunk; the refill of the stage read in
//    the previous chunk is issued right after it, NSTAGE-1 chunks ahead;
//  * kSyncRing: each warp arrives on the stage's "empty" mbarrier, and the
//    producer refills a stage one chunk behind the consumers, so warps run
//    decoupled without block-wide barriers.
// Per-lane df sums are reduced across the warp with a fixed shuffle tree in
// df arithmetic, converted to FP64 once, and combined by the common epilogue.
// Every wait is bounded (kWaitLimit polls, or an abort raised by another
// thread of the block); a block that gives up records kErrPipelineTimeout.
template <int RNW, int RG, int NWC, int NWARP, int KC, int NSTAGE, int SYNC, int GROUP>
__global__ void __launch_bounds__(NWARP * 32)
mixed_noflag_kernel(Problem p, Partials part, SplitPlanes s, int band_begin, int band_end,
                    int row_tiles, int band_tiles) {
    constexpr int BN = NWARP * RNW;            // bands per block
    constexpr int K = BN * RG * NWC * 2;       // doubles in the block result
    constexpr int STAGE = (2 * RG + BN) * KC;  // float4 per stage
    static_assert(KC % 32 == 0, "chunk must be a multiple of the warp width");
    static_assert(NSTAGE >= 2, "need at least two stages");
    extern __shared__ __align__(128) float4 stage_mem[];
    __shared__ unsigned long long full_bar[NSTAGE], empty_bar[NSTAGE];
    __shared__ int abort_flag;
    __shared__ double S[K];

    const int tiles_per_group = GROUP * band_tiles;
    const int grp = blockIdx.x / tiles_per_group;
    const int in_grp = blockIdx.x - grp * tiles_per_group;
    const int rows_in_grp = min(GROUP, row_tiles - grp * GROUP);
    const int row_tile = grp * GROUP + in_grp % rows_in_grp;
    const int band_tile = in_grp / rows_in_grp;
    const int row0 = row_tile * RG;
    const int band0 = band_begin + band_tile * BN;
    const int iw0 = blockIdx.y * NWC;
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
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            const size_t r = (size_t)min(row0 + g, p.ng - 1) * nc + k0;
            bulk_copy_g2s(st + g * KC, s.rowW + r, bytes, bar);
            bulk_copy_g2s(st + (RG + g) * KC, s.rowQ + r, bytes, bar);
        }
#pragma unroll
        for (int n = 0; n < BN; ++n) {
            const size_t b = (size_t)min(band0 + n, band_end - 1) * nc + k0;
            bulk_copy_g2s(st + (2 * RG + n) * KC, s.band + b, bytes, bar);
        }
    };

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int i = 0; i < NSTAGE; ++i) {
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
#pragma unroll
    for (int n = 0; n < RNW; ++n) {
        const int b = min(bandw + n, band_end - 1);
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            const float2 x = s.wx[(size_t)b * p.nw + min(iw0 + w, p.nw - 1)];
            wx[n][w] = {x.x, x.y};
            pole_thr[n][w] = 1e-6f * x.x * x.x;  // |wdiff|^2 < (1e-3 |wx|)^2
        }
    }
    df acc[RNW][RG][NWC][2];
#pragma unroll
    for (int n = 0; n < RNW; ++n)
#pragma unroll
        for (int g = 0; g < RG; ++g)
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                acc[n][g][w][0] = {0.f, 0.f};
                acc[n][g][w][1] = {0.f, 0.f};
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
        const int sidx = c % NSTAGE;
        const bool ok = mbar_wait(&full_bar[sidx], (unsigned)((c / NSTAGE) & 1), abort);
        if (ok) {
            const float4 *st = stage_mem + sidx * STAGE;      // row planes
            const float4 *sb = st + (2 * RG + warp * RNW) * KC;  // this warp's bands
            const int k0 = c * KC;
            const int cnt = min(KC, nc - k0);
#pragma unroll 1
            for (int il = lane; il < cnt; il += 32)
                mixed_column<RNW, RG, NWC, KC>(p, st, sb, il, k0 + il, row0, bandw, band_end,
                                               iw0, wx, pole_thr, acc);
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
        return;
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
                    df v = acc[n][g][w][ri];
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
    noflag_epilogue<BN, RG, NWC>(p, part, S, row0, band0, band_end, iw0,
                                 (long long)band_tile * row_tiles + row_tile, row_tile);
}

constexpr int kGroup = 16;
constexpr int kWarps = 4;

// Compiled pipeline variants of the mixed kernel (the autotuner picks one).
struct MixedVariant {
    int kc, stages, sync;
    const char *name;
};
constexpr MixedVariant kMixedVariants[] = {
    {128, 2, kSyncBlock, "block-sync, 2 x 128 columns"},
    {128, 3, kSyncBlock, "block-sync, 3 x 128 columns"},
    {128, 2, kSyncRing, "mbarrier ring, 2 x 128 columns"},
    {64, 4, kSyncRing, "mbarrier ring, 4 x 64 columns"},
};
constexpr int kNumMixedVariants = sizeof(kMixedVariants) / sizeof(kMixedVariants[0]);

template <int RNW, int RG, int NWC, int KC, int NSTAGE, int SYNC>
cudaError_t launch_mixed_t(const Problem &p, const Partials &part, const SplitPlanes &s, int b0,
                           int b1, cudaStream_t st) {
    constexpr int BN = kWarps * RNW;
    const int row_tiles = ceil_div(p.ng, RG), band_tiles = ceil_div(b1 - b0, BN);
    const size_t smem = sizeof(float4) * NSTAGE * (2 * RG + BN) * KC;
    auto kern = mixed_noflag_kernel<RNW, RG, NWC, kWarps, KC, NSTAGE, SYNC, kGroup>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((unsigned)row_tiles * band_tiles, ceil_div(p.nw, NWC));
    kern<<<grid, kWarps * 32, smem, st>>>(p, part, s, b0, b1, row_tiles, band_tiles);
    count_launch();
    return cudaGetLastError();
}

template <int RNW, int RG, int NWC>
cudaError_t launch_mixed_variant(int v, const Problem &p, const Partials &part,
                                 const SplitPlanes &s, int b0, int b1, cudaStream_t st) {
    switch (v) {
        case 0: return launch_mixed_t<RNW, RG, NWC, 128, 2, kSyncBlock>(p, part, s, b0, b1, st);
        case 2: return launch_mixed_t<RNW, RG, NWC, 128, 2, kSyncRing>(p, part, s, b0, b1, st);
        case 3: return launch_mixed_t<RNW, RG, NWC, 64, 4, kSyncRing>(p, part, s, b0, b1, st);
        default: return launch_mixed_t<RNW, RG, NWC, 128, 3, kSyncBlock>(p, part, s, b0, b1, st);
    }
}

}  // namespace

static int nwc_for(int nw) { return nw <= 4 ? nw : 8; }

// Rows per block for a frequency chunk: 2 rows x 4 frequencies keeps the df
// accumulators (RG * NWC * 2 values of 2 floats) within ~100 registers.
static int mixed_rg(int nwc) { return nwc <= 4 ? 2 : 1; }

TileShape mixed_noflag_shape(const Problem &p) {
    const int nwc = nwc_for(p.nw);
    return TileShape{kWarps, mixed_rg(nwc), nwc, kWarps * 32};
}

int mixed_variant_count() { return kNumMixedVariants; }
const char *mixed_variant_name(int v) {
    return (v >= 0 && v < kNumMixedVariants) ? kMixedVariants[v].name : "default";
}
int mixed_default_variant() { return 1; }

size_t mixed_split_bytes(const Problem &p) {
    return sizeof(float4) * ((size_t)2 * p.ng * p.nc + (size_t)p.nb * p.nc) +
           sizeof(float2) * (size_t)p.nb * p.nw;
}

cudaError_t launch_mixed_noflag(const Problem &p, const Partials &part, void *split_ws, int b0,
                                int b1, cudaStream_t st, int variant) {
    if (b1 <= b0 || p.ng == 0) return cudaSuccess;
    const SplitPlanes s = planes(p, split_ws);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms > 0 ? sms * 8 : 1024;
    split_rows_kernel<<<blocks, 256, 0, st>>>(p, s);
    split_bands_kernel<<<blocks, 256, 0, st>>>(p, s, b0, b1);
    count_launch(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    switch (nwc_for(p.nw)) {
        case 1: return launch_mixed_t<1, 2, 1, 128, 3, kSyncBlock>(p, part, s, b0, b1, st);
        case 2: return launch_mixed_t<1, 2, 2, 128, 3, kSyncBlock>(p, part, s, b0, b1, st);
        case 3: return launch_mixed_variant<1, 2, 3>(variant, p, part, s, b0, b1, st);
        case 4: return launch_mixed_t<1, 2, 4, 128, 3, kSyncBlock>(p, part, s, b0, b1, st);
        default: return launch_mixed_variant<1, 1, 8>(variant, p, part, s, b0, b1, st);
    }
}

}  // namespace gpp

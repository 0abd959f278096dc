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
// the 1e-8 target.  A block's two G' rows are the two lanes of the packed
// f32x2 instructions (gpp_df2.cuh), so a term costs ~45 packed FP32
// instructions instead of ~11 FP64 ones (~700 FP32-equivalents).
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
// Work decomposition: a block owns one row pair x 4 bands x NWC frequencies,
// threads stride over ig, and a grouped tile order keeps GROUP row tiles
// resident in L2 while all band tiles stream past them.
#include "gpp_kernels.h"
#include "gpp_tiles_mixed.cuh"

namespace gpp {

namespace {

size_t row_pair_elems(const Problem &p) { return (size_t)((p.ng + 1) / 2) * 4 * p.nc; }

SplitPlanes planes(const Problem &p, void *ws) {
    SplitPlanes s;
    s.rows = static_cast<float4 *>(ws);
    s.band = s.rows + row_pair_elems(p);
    s.wx = reinterpret_cast<float2 *>(s.band + (size_t)p.nb * p.nc);
    s.masks = reinterpret_cast<unsigned long long *>(s.wx + (size_t)p.nb * p.nw);
    return s;
}

size_t mask_words(const Problem &p) {
    return (size_t)((p.ng + 1) / 2) * ((p.nc + kMaskCols - 1) / kMaskCols);
}

// One thread per (row pair, ig): Q = wtilde * I_eps in FP64 for both rows,
// then the hi/lo splits (split_bits: integer operations, off the FP64 pipe)
// interleaved by row (the row-pair plane layout).  Blocks cover 256 columns
// of one row pair at a time (grid x over columns, y over row pairs).
// The same pass sets the row pairs' value-bucket masks: lanes that share a
// mask word OR their bits together and one of them updates the word (the
// result does not depend on the order).
__global__ void __launch_bounds__(256) split_rows_kernel(Problem p, SplitPlanes s, int pair0,
                                                         int pair1) {
    const size_t nc = (size_t)p.nc;
    const size_t nmw = (nc + kMaskCols - 1) / kMaskCols;
    for (int jj = pair0 + blockIdx.y; jj < pair1; jj += gridDim.y) {
        const size_t j = (size_t)jj;
        const size_t r0 = 2 * j, r1 = min(2 * j + 1, (size_t)p.ng - 1);
        for (size_t ig = (size_t)blockIdx.x * 256 + threadIdx.x; ig < nc;
             ig += (size_t)gridDim.x * 256) {
            const double2 wt0 = __ldg(p.wt + r0 * nc + ig), wt1 = __ldg(p.wt + r1 * nc + ig);
            const double2 q0 = cmul(wt0, __ldg(p.ieps + r0 * nc + ig));
            const double2 q1 = cmul(wt1, __ldg(p.ieps + r1 * nc + ig));
            const df a0 = split_bits(wt0.x), a1 = split_bits(wt1.x);
            const df b0 = split_bits(wt0.y), b1 = split_bits(wt1.y);
            const df c0 = split_bits(q0.x), c1 = split_bits(q1.x);
            const df d0 = split_bits(q0.y), d1 = split_bits(q1.y);
            float4 *o = s.rows + j * 4 * nc + ig;
            o[0] = make_float4(a0.h, a1.h, a0.l, a1.l);
            o[nc] = make_float4(b0.h, b1.h, b0.l, b1.l);
            o[2 * nc] = make_float4(c0.h, c1.h, c0.l, c1.l);
            o[3 * nc] = make_float4(d0.h, d1.h, d0.l, d1.l);
            const unsigned long long bits =
                bucket_bit(bucket_code(a0.h)) | bucket_bit(bucket_code(a1.h));
            const unsigned long long word = j * nmw + ig / kMaskCols;
            const unsigned act = __activemask();
            const unsigned grp = __match_any_sync(act, word);
            const unsigned lo = __reduce_or_sync(grp, (unsigned)bits);
            const unsigned hi = __reduce_or_sync(grp, (unsigned)(bits >> 32));
            if ((int)(threadIdx.x & 31) == __ffs(grp) - 1)
                atomicOr(s.masks + word, ((unsigned long long)hi << 32) | lo);
        }
    }
}

__global__ void __launch_bounds__(256) split_bands_kernel(Problem p, SplitPlanes s, int b0,
                                                          int b1) {
    const size_t n = (size_t)(b1 - b0) * p.nc;
    const size_t base = (size_t)b0 * p.nc;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) {
        const double2 a = __ldg(p.aqsn + base + i);
        const df ar = split_bits(a.x), ai = split_bits(a.y);
        s.band[base + i] = make_float4(ar.h, ar.l, ai.h, ai.l);
    }
    const int nwx = (b1 - b0) * p.nw;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < nwx; i += gridDim.x * 256) {
        const int b = b0 + i / p.nw, iw = i % p.nw;
        const df x = split(__ldg(p.wx + (size_t)b * p.wx_stride + iw));
        s.wx[(size_t)b * p.nw + iw] = make_float2(x.h, x.l);
    }
}

template <int RNW, int RG, int NWC, int NWARP, int KC, int NSTAGE, int SYNC, int GROUP, int MINB>
__global__ void __launch_bounds__(NWARP * 32, MINB)
mixed_noflag_kernel(Problem p, Partials part, SplitPlanes s, int band_begin, int band_end,
                    int row_tile0, int rows_here, int row_tiles, int band_tiles) {
    // Grouped tile order over this launch's row tiles [row_tile0, +rows_here):
    // GROUP consecutive row tiles share each band tile, so a group's row
    // planes stay in L2 while the band tiles stream past.
    const int tiles_per_group = GROUP * band_tiles;
    const int grp = blockIdx.x / tiles_per_group;
    const int in_grp = blockIdx.x - grp * tiles_per_group;
    const int rows_in_grp = min(GROUP, rows_here - grp * GROUP);
    const int row_tile = row_tile0 + grp * GROUP + in_grp % rows_in_grp;
    const int band_tile = in_grp / rows_in_grp;
    mixed_tile<RNW, RG, NWC, NWARP, KC, NSTAGE, SYNC>(
        p, part, s, band_begin, band_end, row_tile, band_tile, blockIdx.y,
        (long long)band_tile * row_tiles + row_tile, false);
}

constexpr int kGroup = 16;
constexpr int kWarps = 4;

// Compiled variants of the mixed kernel (the autotuner picks one): the tile
// shape -- `warps` warps per block, each owning `rnw` bands of the block's
// row pair, so warps x rnw bands x 2 rows per block -- and the shared-memory
// pipeline (chunk width, stage count, recycling).  `minb` is the
// __launch_bounds__ minimum of resident blocks per SM: 0 leaves the register
// count to the compiler's default heuristic (a minimum of 1 would let it
// take up to 255), 5 caps it at 96 registers.  The shape sets the block
// partials' layout (and so the order of the final sums): variants of one
// shape give identical bits, other shapes agree to rounding.
struct MixedVariant {
    int kc, stages, sync, minb, warps, rnw;
    const char *name;
};
constexpr MixedVariant kMixedVariants[] = {
    {128, 2, kSyncBlock, 0, 4, 1, "4 bands x 2 rows, block-sync, 2 x 128 columns"},
    {128, 3, kSyncBlock, 0, 4, 1, "4 bands x 2 rows, block-sync, 3 x 128 columns"},
    {128, 2, kSyncRing, 0, 4, 1, "4 bands x 2 rows, mbarrier ring, 2 x 128 columns"},
    {64, 4, kSyncRing, 0, 4, 1, "4 bands x 2 rows, mbarrier ring, 4 x 64 columns"},
    {128, 2, kSyncBlock, 5, 4, 1, "4 bands x 2 rows, block-sync, 2 x 128 columns, 5 blocks/SM"},
    {128, 3, kSyncRing, 0, 4, 1, "4 bands x 2 rows, mbarrier ring, 3 x 128 columns"},
    {192, 2, kSyncBlock, 0, 4, 1, "4 bands x 2 rows, block-sync, 2 x 192 columns"},
    {256, 2, kSyncBlock, 0, 4, 1, "4 bands x 2 rows, block-sync, 2 x 256 columns"},
    {192, 2, kSyncBlock, 0, 8, 1, "8 bands x 2 rows (8 warps), block-sync, 2 x 192 columns"},
    {256, 2, kSyncBlock, 0, 8, 1, "8 bands x 2 rows (8 warps), block-sync, 2 x 256 columns"},
    {192, 2, kSyncBlock, 3, 4, 2, "8 bands x 2 rows (2 bands per warp), block-sync, 2 x 192 columns"},
};
constexpr int kNumMixedVariants = sizeof(kMixedVariants) / sizeof(kMixedVariants[0]);

// Frequency chunks compiled in every variant: 3 (the workloads' grids) and
// 8 (large grids); chunks of 1, 2 and 4 frequencies have one kernel, of
// the 4 bands x 2 rows shape.  Two bands per warp double the accumulators:
// that shape is compiled for 3 frequencies only (8 would spill heavily).
bool variant_compiled(int v, int nwc) {
    if (v < 0 || v >= kNumMixedVariants) return false;
    const MixedVariant &m = kMixedVariants[v];
    if (nwc != 3 && nwc != 8) return m.warps == kWarps && m.rnw == 1;
    return !(m.rnw == 2 && nwc > 4);
}

template <int RNW, int RG, int NWC, int KC, int NSTAGE, int SYNC, int MINB = 0, int NWARP = kWarps>
cudaError_t launch_mixed_t(const Problem &p, const Partials &part, const SplitPlanes &s, int b0,
                           int b1, RowTiles rt, cudaStream_t st) {
    constexpr int BN = NWARP * RNW;
    const int row_tiles = ceil_div(p.ng, RG), band_tiles = ceil_div(b1 - b0, BN);
    const RowTiles r = rt.clip(row_tiles);
    if (r.end <= r.begin) return cudaSuccess;
    const size_t smem = sizeof(float4) * NSTAGE * (2 * RG + BN) * KC;
    // The 8-frequency tile holds 64 accumulator registers: keep it at three
    // resident blocks unless the variant asks for more.
    constexpr int kMinB = MINB ? MINB : (NWC > 4 ? 3 : 0);
    auto kern = mixed_noflag_kernel<RNW, RG, NWC, NWARP, KC, NSTAGE, SYNC, kGroup, kMinB>;
    // Opt in to the full dynamic size (the default cap is 48 KB including
    // the kernel's static shared memory).
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)(r.end - r.begin) * band_tiles, ceil_div(p.nw, NWC));
    kern<<<grid, NWARP * 32, smem, st>>>(p, part, s, b0, b1, r.begin, r.end - r.begin, row_tiles,
                                         band_tiles);
    count_launch();
    return cudaGetLastError();
}

template <int RG, int NWC>
cudaError_t launch_mixed_variant(int v, const Problem &p, const Partials &part,
                                 const SplitPlanes &s, int b0, int b1, RowTiles rt,
                                 cudaStream_t st) {
    switch (v) {
        case 0: return launch_mixed_t<1, RG, NWC, 128, 2, kSyncBlock>(p, part, s, b0, b1, rt, st);
        case 2: return launch_mixed_t<1, RG, NWC, 128, 2, kSyncRing>(p, part, s, b0, b1, rt, st);
        case 3: return launch_mixed_t<1, RG, NWC, 64, 4, kSyncRing>(p, part, s, b0, b1, rt, st);
        case 4:
            return launch_mixed_t<1, RG, NWC, 128, 2, kSyncBlock, 5>(p, part, s, b0, b1, rt, st);
        case 5: return launch_mixed_t<1, RG, NWC, 128, 3, kSyncRing>(p, part, s, b0, b1, rt, st);
        case 6: return launch_mixed_t<1, RG, NWC, 192, 2, kSyncBlock>(p, part, s, b0, b1, rt, st);
        case 7: return launch_mixed_t<1, RG, NWC, 256, 2, kSyncBlock>(p, part, s, b0, b1, rt, st);
        case 8:
            return launch_mixed_t<1, RG, NWC, 192, 2, kSyncBlock, 0, 8>(p, part, s, b0, b1, rt, st);
        case 9:
            return launch_mixed_t<1, RG, NWC, 256, 2, kSyncBlock, 0, 8>(p, part, s, b0, b1, rt, st);
        case 10:
            if constexpr (NWC <= 4)
                return launch_mixed_t<2, RG, NWC, 192, 2, kSyncBlock, 3>(p, part, s, b0, b1, rt, st);
            else
                return cudaErrorInvalidValue;
        default:
            return launch_mixed_t<1, RG, NWC, 128, 3, kSyncBlock>(p, part, s, b0, b1, rt, st);
    }
}

}  // namespace

static int nwc_for(int nw) { return nw <= 4 ? nw : 8; }

// Rows per block: one row pair of the split planes, the two lanes of the
// packed df2 arithmetic.
static int mixed_rg(int) { return 2; }

TileShape mixed_noflag_shape(const Problem &p, int variant) {
    const int nwc = nwc_for(p.nw);
    const MixedVariant &v =
        kMixedVariants[variant_compiled(variant, nwc) ? variant : mixed_default_variant()];
    return TileShape{v.warps * v.rnw, mixed_rg(nwc), nwc, v.warps * 32};
}

bool mixed_variant_valid(int variant, int nw) { return variant_compiled(variant, nwc_for(nw)); }

int mixed_variant_count() { return kNumMixedVariants; }
const char *mixed_variant_name(int v) {
    return (v >= 0 && v < kNumMixedVariants) ? kMixedVariants[v].name : "default";
}
// Block-sync with 192-column chunks: the fastest at 3 frequencies and within
// 1% of the fastest at 32 on GB300.
int mixed_default_variant() { return 6; }

size_t mixed_split_bytes(const Problem &p) {
    return sizeof(float4) * (row_pair_elems(p) + (size_t)p.nb * p.nc) +
           sizeof(float2) * (size_t)p.nb * p.nw + sizeof(unsigned long long) * mask_words(p);
}

SplitPlanes split_planes_at(const Problem &p, void *split_ws) { return planes(p, split_ws); }

static int split_blocks() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms * 8 : 1024;
}

cudaError_t launch_split_bands(const Problem &p, void *split_ws, int b0, int b1, cudaStream_t st) {
    const SplitPlanes s = planes(p, split_ws);
    cudaError_t e = cudaMemsetAsync(s.masks, 0, sizeof(unsigned long long) * mask_words(p), st);
    if (e != cudaSuccess) return e;
    split_bands_kernel<<<split_blocks(), 256, 0, st>>>(p, s, b0, b1);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_rows(const Problem &p, void *split_ws, RowTiles pairs, cudaStream_t st) {
    const RowTiles r = pairs.clip((p.ng + 1) / 2);
    if (r.end <= r.begin) return cudaSuccess;
    // Columns: up to 64 blocks of 256 per row pair; row pairs: enough blocks
    // in y for ~8 per SM in all.
    const int bx = std::min(64, std::max(1, ceil_div(p.nc, 256)));
    const int by = std::min(r.end - r.begin, std::max(1, split_blocks() / bx));
    split_rows_kernel<<<dim3(bx, by), 256, 0, st>>>(p, planes(p, split_ws), r.begin, r.end);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split(const Problem &p, void *split_ws, int b0, int b1, cudaStream_t st) {
    cudaError_t e = launch_split_bands(p, split_ws, b0, b1, st);
    if (e == cudaSuccess) e = launch_split_rows(p, split_ws, RowTiles(), st);
    return e;
}

// Three resident blocks (at most 168 registers) for up to 4 frequencies:
// the occupied-band kernel is latency-bound, and the third block beat the
// compiler's 222-register choice by 15% (4 blocks spilled and lost).
template <int RG, int NWC, int THREADS, int SEM>
__global__ void __launch_bounds__(THREADS, NWC <= 4 ? 3 : 2)
flag_mixed_kernel(Problem p, Partials part, SplitPlanes s, int row_tile0, int count,
                  int row_tiles, int *next) {
    constexpr int K = RG * NWC * 4;
    __shared__ double red[(THREADS / 32) * K];
    __shared__ double S[K];
    __shared__ int item;
    if (!next) {
        const int row_tile = row_tile0 + blockIdx.x;
        flag_mixed_tile<RG, NWC, THREADS, SEM>(p, part, s, row_tile, blockIdx.y, blockIdx.z,
                                               (long long)blockIdx.y * row_tiles + row_tile, red,
                                               S);
        return;
    }
    // Persistent grid beside the tensor-core GEMM: (row tile, band, chunk)
    // items from the counter, each computed and written as in the grid above.
    const long long items = (long long)count * p.nv * ((p.nw + NWC - 1) / NWC);
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(next, 1);
        __syncthreads();
        const long long it = item;
        if (it >= items) break;
        const int row_tile = row_tile0 + (int)(it % count);
        const long long rest = it / count;
        const int band = (int)(rest % p.nv);
        flag_mixed_tile<RG, NWC, THREADS, SEM>(p, part, s, row_tile, band, (int)(rest / p.nv),
                                               (long long)band * row_tiles + row_tile, red, S);
        __syncthreads();  // S read by the epilogue, `item` by every thread, before reuse
    }
}

template <int NWC>
cudaError_t launch_flag_mixed_t(const Problem &p, const Partials &part, const SplitPlanes &s,
                                RowTiles rt, int blocks_per_sm, int *next, cudaStream_t st) {
    const int row_tiles = ceil_div(p.ng, 2);
    const RowTiles r = rt.clip(row_tiles);
    if (r.end <= r.begin) return cudaSuccess;
    const int count = r.end - r.begin;
    dim3 grid(count, p.nv, ceil_div(p.nw, NWC));
    // The counter is a 32-bit int: past 2^30 items the one-tile grid instead.
    const long long items = (long long)count * grid.y * grid.z;
    const int per_sm = next && items < (1ll << 30) ? flag_blocks_per_sm(blocks_per_sm) : 0;
    if (per_sm > 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = dim3((unsigned)std::max(1ll, std::min<long long>(items, (long long)std::max(sms, 1) * per_sm)));
        const cudaError_t e = cudaMemsetAsync(next, 0, sizeof(int), st);
        if (e != cudaSuccess) return e;
    } else {
        next = nullptr;
    }
    if (p.semantics == kSemKerSeq) {
        prefer_max_shared(flag_mixed_kernel<2, NWC, 128, kSemKerSeq>);
        flag_mixed_kernel<2, NWC, 128, kSemKerSeq><<<grid, 128, 0, st>>>(p, part, s, r.begin,
                                                                        count, row_tiles, next);
    } else {
        prefer_max_shared(flag_mixed_kernel<2, NWC, 128, kSemComplexSeq>);
        flag_mixed_kernel<2, NWC, 128, kSemComplexSeq><<<grid, 128, 0, st>>>(
            p, part, s, r.begin, count, row_tiles, next);
    }
    count_launch();
    return cudaGetLastError();
}

// Self-test of the bounded pipeline wait: one block waits on an mbarrier
// that nothing arrives at, gives up after `polls` polls and records
// kErrPipelineTimeout exactly as a tile does, then returns.
__global__ void __launch_bounds__(32) wait_selftest_kernel(int *err, int polls) {
    __shared__ unsigned long long bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        abort_flag = 0;
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    const bool ok = mbar_wait(&bar, 0u, &abort_flag, polls);
    __syncwarp();
    if (threadIdx.x == 0) {
        if (!ok) atomicOr(err, kErrPipelineTimeout);
        mbar_inval(&bar);
    }
}

cudaError_t launch_wait_selftest(int *err, int polls, cudaStream_t st) {
    wait_selftest_kernel<<<1, 32, 0, st>>>(err, polls);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_flag_mixed(const Problem &p, const Partials &part, void *split_ws,
                              cudaStream_t st, RowTiles rt, int blocks_per_sm, int *next) {
    if (p.nv <= 0 || p.ng == 0) return cudaSuccess;
    const SplitPlanes s = planes(p, split_ws);
    switch (nwc_for(p.nw)) {
        case 1: return launch_flag_mixed_t<1>(p, part, s, rt, blocks_per_sm, next, st);
        case 2: return launch_flag_mixed_t<2>(p, part, s, rt, blocks_per_sm, next, st);
        case 3: return launch_flag_mixed_t<3>(p, part, s, rt, blocks_per_sm, next, st);
        case 4: return launch_flag_mixed_t<4>(p, part, s, rt, blocks_per_sm, next, st);
        default: return launch_flag_mixed_t<8>(p, part, s, rt, blocks_per_sm, next, st);
    }
}

cudaError_t launch_mixed_noflag(const Problem &p, const Partials &part, void *split_ws, int b0,
                                int b1, cudaStream_t st, int variant, RowTiles rt) {
    if (b1 <= b0 || p.ng == 0) return cudaSuccess;
    const SplitPlanes s = planes(p, split_ws);
    switch (nwc_for(p.nw)) {
        case 1: return launch_mixed_t<1, 2, 1, 128, 3, kSyncBlock>(p, part, s, b0, b1, rt, st);
        case 2: return launch_mixed_t<1, 2, 2, 128, 3, kSyncBlock>(p, part, s, b0, b1, rt, st);
        case 3: return launch_mixed_variant<2, 3>(variant, p, part, s, b0, b1, rt, st);
        case 4: return launch_mixed_t<1, 2, 4, 128, 3, kSyncBlock>(p, part, s, b0, b1, rt, st);
        default: return launch_mixed_variant<2, 8>(variant, p, part, s, b0, b1, rt, st);
    }
}

}  // namespace gpp

// gpp_fp64.cu -- FP64 CUDA-core kernels of the GPP sigma reduction for
// sm_103a (one state per launch), the deterministic fixed-order reduction,
// the static term, and the FMA throughput probe.  The tile bodies and the
// algorithm notes live in gpp_tiles_fp64.cuh.  On GB300 the FP64 pipe
// retires ~2 DFMA/clk/SM, so the unoccupied-band kernel is bound by FP64
// issue, not by HBM (~16 B per (n1,igp,ig) triple against ~34 FP64
// instructions).  No floating-point atomics anywhere: results are
// bit-reproducible.
#include <cstdio>

#include <algorithm>
#include <cstdlib>

#include "gpp_kernels.h"
#include "gpp_tiles_fp64.cuh"

namespace gpp {

namespace {

// Row tiles per group of the tile order: a group's G' rows (16 row pairs,
// 32 MB at ncouls 32768) stay in L2 while every band tile streams past
// them, so each row is read from HBM about once per launch and each band
// once per group, instead of every row once per band tile.
constexpr int kFp64Group = 16;

template <int RN, int RG, int NWC, int THREADS>
__global__ void __launch_bounds__(THREADS)
noflag_fp64_kernel(Problem p, Partials part, int band_begin, int band_end, int row_tile0,
                   int rows_here, int row_tiles, int band_tiles) {
    constexpr int K = RN * RG * NWC * 2;
    __shared__ double red[(THREADS / 32) * K];
    __shared__ double S[K];
    // Grouped order over this launch's row tiles [row_tile0, +rows_here).
    const int tiles_per_group = kFp64Group * band_tiles;
    const int grp = blockIdx.x / tiles_per_group;
    const int in_grp = blockIdx.x - grp * tiles_per_group;
    const int rows_in_grp = min(kFp64Group, rows_here - grp * kFp64Group);
    const int row_tile = row_tile0 + grp * kFp64Group + in_grp % rows_in_grp;
    const int band_tile = in_grp / rows_in_grp;
    noflag_fp64_tile<RN, RG, NWC, THREADS>(p, part, band_begin, band_end, row_tile, band_tile,
                                           blockIdx.y, (long long)band_tile * row_tiles + row_tile,
                                           red, S);
}

template <int RG, int NWC, int THREADS, int SEM>
__global__ void __launch_bounds__(THREADS)
flag_fp64_kernel(Problem p, Partials part, int row_tile0, int row_tiles) {
    constexpr int K = RG * NWC * 4;
    __shared__ double red[(THREADS / 32) * K];
    __shared__ double S[K];
    const int row_tile = row_tile0 + blockIdx.x;
    flag_fp64_tile<RG, NWC, THREADS, SEM>(p, part, row_tile, blockIdx.y, blockIdx.z,
                                          (long long)blockIdx.y * row_tiles + row_tile, red, S);
}

// Band-independent frequencies: blockIdx.y covers NB occupied bands and
// blockIdx.z a frequency chunk, blockIdx.x one of `count` row tiles from
// row_tile0.  With `next` set, a persistent grid instead: each block takes
// (row tile, band group, chunk) items from the counter until none is left,
// so blocks that share an SM take fewer; every item is computed and written
// as in the one-tile grid, so the bits do not depend on the grid.
template <int RG, int NWC, int NB, int THREADS, int SEM>
__global__ void __launch_bounds__(THREADS)
flag_fp64_multi_kernel(Problem p, Partials part, int row_tile0, int count, int row_tiles,
                       int *next) {
    constexpr int K = NB * RG * NWC * 4;
    __shared__ double red[(THREADS / 32) * K];
    __shared__ double S[K];
    __shared__ int item;
    if (!next) {
        flag_fp64_multi_tile<RG, NWC, NB, THREADS, SEM>(p, part, row_tile0 + blockIdx.x,
                                                        blockIdx.y * NB, blockIdx.z, row_tiles,
                                                        red, S);
        return;
    }
    const int groups = (p.nv + NB - 1) / NB;
    const long long items = (long long)count * groups * ((p.nw + NWC - 1) / NWC);
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(next, 1);
        __syncthreads();
        const long long it = item;
        if (it >= items) break;
        const int t = (int)(it % count);
        const long long rest = it / count;
        flag_fp64_multi_tile<RG, NWC, NB, THREADS, SEM>(p, part, row_tile0 + t,
                                                        (int)(rest % groups) * NB,
                                                        (int)(rest / groups), row_tiles, red, S);
        __syncthreads();  // S read by the epilogue, `item` by every thread, before reuse
    }
}

// Static term of reduce_achstemp (gppComplex_seq.cpp:66-101): one thread per
// (n1, my_igp) pair; each block leaves one partial.
__global__ void __launch_bounds__(256) achstemp_kernel(Problem p, double2 *partials, int *err) {
    __shared__ double red[8 * 2];
    __shared__ double S[2];
    const long long npairs = (long long)p.nb * p.ng;
    const long long pr = (long long)blockIdx.x * 256 + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (pr < npairs) {
        const int n1 = (int)(pr / p.ng), my_igp = (int)(pr % p.ng);
        const int igp = resolve_igp(p, my_igp, err);
        if (igp >= 0) {
            const double2 m = __ldg(p.aqsm + (size_t)n1 * p.nc + igp);
            const double2 an = __ldg(p.aqsn + (size_t)n1 * p.nc + igp);
            const double2 ie = __ldg(p.ieps + (size_t)my_igp * p.nc + igp);
            const double2 schs = make_double2(-ie.x, -ie.y);
            const double2 matng = cmul(an, make_double2(m.x, -m.y));
            if (sqrt(schs.x * schs.x + schs.y * schs.y) > kTo1) {
                const double2 c = cscale(cmul(matng, schs), __ldg(p.vcoul + igp) * 0.5);
                v[0] = c.x;
                v[1] = c.y;
            }
        }
    }
    block_reduce<2, 256>(v, red, S);
    if (threadIdx.x == 0) partials[blockIdx.x] = make_double2(S[0], S[1]);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS)
reduce_kernel(const double2 *src, long long stride, int len, ReduceOut out) {
    __shared__ double red[(THREADS / 32) * 2];
    __shared__ double S[2];
    const double2 *seg = src + (long long)blockIdx.x * stride;
    double v[2] = {0.0, 0.0};
    for (int t = threadIdx.x; t < len; t += THREADS) {
        const double2 x = seg[t];
        v[0] += x.x;
        v[1] += x.y;
    }
    block_reduce<2, THREADS>(v, red, S);
    if (threadIdx.x == 0) {
        const int s = blockIdx.x;
        if (out.c) {
            double2 r = make_double2(S[0], S[1]);
            if (out.accumulate) r = cadd(out.c[s], r);
            out.c[s] = r;
        }
        if (out.re) out.re[s] += S[0];
        if (out.im) out.im[s] += S[1];
    }
}

template <int RN, int RG, int NWC, int THREADS>
cudaError_t launch_noflag_t(const Problem &p, const Partials &part, int b0, int b1, RowTiles rt,
                            cudaStream_t s) {
    const int row_tiles = ceil_div(p.ng, RG);
    const RowTiles r = rt.clip(row_tiles);
    if (r.end <= r.begin) return cudaSuccess;
    const int band_tiles = ceil_div(b1 - b0, RN);
    dim3 grid((unsigned)((long long)(r.end - r.begin) * band_tiles), ceil_div(p.nw, NWC));
    noflag_fp64_kernel<RN, RG, NWC, THREADS><<<grid, THREADS, 0, s>>>(
        p, part, b0, b1, r.begin, r.end - r.begin, row_tiles, band_tiles);
    count_launch();
    return cudaGetLastError();
}

// Occupied bands in pairs when the frequencies are band-independent (the
// solver once per pair; the same bits).  GPP_FLAG_MULTI=0 keeps one band per
// block, read on every call.
bool flag_multi_enabled() {
    const char *v = getenv("GPP_FLAG_MULTI");
    return !(v && v[0] == '0');
}

template <int RG, int NWC, int NB, int THREADS>
cudaError_t launch_flag_multi_t(const Problem &p, const Partials &part, RowTiles r, int row_tiles,
                                int blocks_per_sm, int *next, cudaStream_t s) {
    const int count = r.end - r.begin;
    dim3 grid(count, ceil_div(p.nv, NB), ceil_div(p.nw, NWC));
    // The counter is a 32-bit int: past 2^30 items the one-tile grid instead.
    const long long items = (long long)count * grid.y * grid.z;
    const int per_sm = next && items < (1ll << 30) ? flag_blocks_per_sm(blocks_per_sm) : 0;
    if (per_sm > 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = dim3((unsigned)std::max(1ll, std::min<long long>(items, (long long)std::max(sms, 1) * per_sm)));
        const cudaError_t e = cudaMemsetAsync(next, 0, sizeof(int), s);
        if (e != cudaSuccess) return e;
    } else {
        next = nullptr;
    }
    if (p.semantics == kSemKerSeq) {
        prefer_max_shared(flag_fp64_multi_kernel<RG, NWC, NB, THREADS, kSemKerSeq>);
        flag_fp64_multi_kernel<RG, NWC, NB, THREADS, kSemKerSeq><<<grid, THREADS, 0, s>>>(
            p, part, r.begin, count, row_tiles, next);
    } else {
        prefer_max_shared(flag_fp64_multi_kernel<RG, NWC, NB, THREADS, kSemComplexSeq>);
        flag_fp64_multi_kernel<RG, NWC, NB, THREADS, kSemComplexSeq><<<grid, THREADS, 0, s>>>(
            p, part, r.begin, count, row_tiles, next);
    }
    count_launch();
    return cudaGetLastError();
}

template <int RG, int NWC, int THREADS>
cudaError_t launch_flag_t(const Problem &p, const Partials &part, RowTiles rt, int blocks_per_sm,
                          int *next, cudaStream_t s) {
    const int row_tiles = ceil_div(p.ng, RG);
    const RowTiles r = rt.clip(row_tiles);
    if (r.end <= r.begin) return cudaSuccess;
    if constexpr (NWC <= 4) {  // two bands of 8 frequencies would spill
        if (p.wx_stride == 0 && p.nv >= 2 && flag_multi_enabled())
            return launch_flag_multi_t<RG, NWC, 2, THREADS>(p, part, r, row_tiles, blocks_per_sm,
                                                            next, s);
    }
    dim3 grid(r.end - r.begin, p.nv, ceil_div(p.nw, NWC));
    if (p.semantics == kSemKerSeq) {
        prefer_max_shared(flag_fp64_kernel<RG, NWC, THREADS, kSemKerSeq>);
        flag_fp64_kernel<RG, NWC, THREADS, kSemKerSeq><<<grid, THREADS, 0, s>>>(p, part, r.begin,
                                                                                row_tiles);
    } else {
        prefer_max_shared(flag_fp64_kernel<RG, NWC, THREADS, kSemComplexSeq>);
        flag_fp64_kernel<RG, NWC, THREADS, kSemComplexSeq><<<grid, THREADS, 0, s>>>(
            p, part, r.begin, row_tiles);
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace

int flag_blocks_per_sm(int asked) {
    const char *v = getenv("GPP_FLAG_BLOCKS_PER_SM");
    return v ? atoi(v) : asked;
}

// Frequencies per block: a whole small frequency grid stays in registers; a
// large grid (e.g. 32 frequencies) is split into chunks of 8.
static int nwc_for(int nw) { return nw <= 4 ? nw : 8; }

TileShape fp64_noflag_shape(const Problem &p) {
    const int nwc = nwc_for(p.nw);
    return nwc <= 4 ? TileShape{4, 2, nwc, 128} : TileShape{2, 2, nwc, 128};
}

TileShape flag_shape(const Problem &p) { return TileShape{1, 2, nwc_for(p.nw), 128}; }

cudaError_t launch_noflag_fp64(const Problem &p, const Partials &part, int b0, int b1,
                               cudaStream_t s, RowTiles rt) {
    if (b1 <= b0 || p.ng == 0) return cudaSuccess;
    switch (nwc_for(p.nw)) {
        case 1: return launch_noflag_t<4, 2, 1, 128>(p, part, b0, b1, rt, s);
        case 2: return launch_noflag_t<4, 2, 2, 128>(p, part, b0, b1, rt, s);
        case 3: return launch_noflag_t<4, 2, 3, 128>(p, part, b0, b1, rt, s);
        case 4: return launch_noflag_t<4, 2, 4, 128>(p, part, b0, b1, rt, s);
        default: return launch_noflag_t<2, 2, 8, 128>(p, part, b0, b1, rt, s);
    }
}

cudaError_t launch_flag_fp64(const Problem &p, const Partials &part, cudaStream_t s, RowTiles rt,
                             int blocks_per_sm, int *next) {
    if (p.nv <= 0 || p.ng == 0) return cudaSuccess;
    switch (nwc_for(p.nw)) {
        case 1: return launch_flag_t<2, 1, 128>(p, part, rt, blocks_per_sm, next, s);
        case 2: return launch_flag_t<2, 2, 128>(p, part, rt, blocks_per_sm, next, s);
        case 3: return launch_flag_t<2, 3, 128>(p, part, rt, blocks_per_sm, next, s);
        case 4: return launch_flag_t<2, 4, 128>(p, part, rt, blocks_per_sm, next, s);
        default: return launch_flag_t<2, 8, 128>(p, part, rt, blocks_per_sm, next, s);
    }
}

int achstemp_blocks(const Problem &p) { return ceil_div((long long)p.nb * p.ng, 256); }

cudaError_t launch_achstemp(const Problem &p, double2 *partials, int *err, cudaStream_t s) {
    const int blocks = achstemp_blocks(p);
    if (blocks == 0) return cudaSuccess;
    achstemp_kernel<<<blocks, 256, 0, s>>>(p, partials, err);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_reduce(const double2 *src, long long stride, int len, int nseg, ReduceOut out,
                          cudaStream_t s) {
    if (nseg <= 0) return cudaSuccess;
    reduce_kernel<512><<<nseg, 512, 0, s>>>(src, stride, len, out);
    count_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FMA throughput probe: independent FMA chains, enough warps to fill the SMs.
namespace {
// Host-to-device transfer by the SMs: each thread streams 16-byte words
// from host memory the device can address (pinned, mapped into the device's
// address space) into device memory, over NVLink-C2C on GB300.  The alternative to a copy-engine
// cudaMemcpyAsync for the host path (gpp_sigma_host); `bytes` is a multiple
// of 16 and both pointers are 16-byte aligned (the caller checks).
__global__ void __launch_bounds__(256) host_pull_kernel(uint4 *__restrict__ dst,
                                                        const uint4 *__restrict__ src,
                                                        size_t words) {
    const size_t stride = (size_t)gridDim.x * 256;
    size_t i = (size_t)blockIdx.x * 256 + threadIdx.x;
    // Four independent 16-byte loads in flight per thread: host memory is a
    // microsecond away.
    for (; i + 3 * stride < words; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride],
                    d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < words; i += stride) dst[i] = src[i];
}


template <typename T, int CHAINS>
__global__ void __launch_bounds__(256) fma_probe_kernel(const T *in, T *out, int iters) {
    T a[CHAINS];
    const T b = in[0], c = in[1];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = in[2 + k] + (T)threadIdx.x;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = fma(a[k], b, c);
    T s = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
cudaError_t time_probe(int blocks, int iters, double *tflops) {
    constexpr int CHAINS = 8;
    T *in = nullptr, *out = nullptr;
    cudaError_t e = cudaMalloc(&in, 16 * sizeof(T));
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&out, (size_t)blocks * 256 * sizeof(T));
    if (e != cudaSuccess) { cudaFree(in); return e; }
    T h[16];
    for (int i = 0; i < 16; ++i) h[i] = (T)(1.0 + 1e-7 * i);
    h[0] = (T)0.999999;
    h[1] = (T)1e-6;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    e = cudaMemcpy(in, h, sizeof(h), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        fma_probe_kernel<T, CHAINS><<<blocks, 256>>>(in, out, iters / 8);  // warm-up
        count_launch();
        cudaEventRecord(e0);
        fma_probe_kernel<T, CHAINS><<<blocks, 256>>>(in, out, iters);
        count_launch();
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && ms > 0.f)
            *tflops = 2.0 * blocks * 256.0 * CHAINS * (double)iters / (ms * 1e-3) * 1e-12;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(in);
    cudaFree(out);
    return e;
}
}  // namespace

cudaError_t probe_fma_peaks(double *fp64_tflops, double *fp32_tflops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = sms * 8;
    e = time_probe<double>(blocks, 4096, fp64_tflops);
    if (e == cudaSuccess) e = time_probe<float>(blocks, 65536, fp32_tflops);
    return e;
}

cudaError_t launch_host_pull(void *dst, const void *src_dev, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // Blocks per SM: GPP_HOST_PULL_BLOCKS (1..16), default 1.  One block of
    // 256 threads per SM, four 16-byte loads in flight per thread, keeps
    // ~2.5 MB in flight -- enough for the link -- and leaves the most room to
    // the computation running beside the pull (GB300, production shape:
    // 221.3 ms per host-path call with 1 block per SM, 224.4 ms with 4).
    static const int per_sm = [] {
        const char *v = getenv("GPP_HOST_PULL_BLOCKS");
        const int k = v ? atoi(v) : 1;
        return (k >= 1 && k <= 16) ? k : 1;
    }();
    const size_t words = bytes / 16;
    const size_t want = (words + 255) / 256;
    const int grid = (int)std::min<size_t>(want, (size_t)std::max(1, sms) * per_sm);
    host_pull_kernel<<<grid, 256, 0, s>>>(static_cast<uint4 *>(dst),
                                           static_cast<const uint4 *>(src_dev), words);
    count_launch();
    return cudaGetLastError();
}

}  // namespace gpp

// gpp_gemm.cu -- unoccupied bands with band-independent frequencies, FP64,
// through one complex GEMM.
//
// With wx the same for every band (the reference's wx_array[nend-nstart],
// gppCudaVer.cpp:389-399 via GPPComplex.cu:406-433), the unoccupied term's
// frequency factor M_iw[r][ig] = Q conj(wdiff) / |wdiff|^2 (Q = wtilde
// I_eps, wdiff = wx_iw - wtilde) depends on the G' row and column only, so
//
//   achtemp[iw] = sum_{r, ig} M_iw[r][ig] G[r][ig],
//   G[r][ig]    = sum_{n1 >= nvband} c[n1][r] aqsn[n1][ig],
//   c[n1][r]    = 0.5 vcoul[igp(r)] conj(aqsm[n1][igp(r)]),
//
// G is one complex GEMM over the bands, and a fused pass over (r, ig) builds
// M on the fly and sums M G per row tile -- the same block-partial slots and
// fixed-order reduction as the per-term kernels.  The per-band output
// acht_n1_loc (iw = 2) needs
//   acht_n1_loc[n1] = sum_r c[n1][r] H[n1][r],  H[n1][r] = sum_ig aqsn[n1][ig] M_2[r][ig],
// a second GEMM against M_2 stored once.  Exact in real arithmetic; only
// the order of the FP64 roundings differs from the per-term kernel.
//
// Both GEMMs are zgemm3m_kernel below, written for GB300's FP64 pipe (no
// library): complex products in the 3M form (Gauss's three real products:
// re = P1 - P2, im = P3 - P1 - P2 with P1 = sum xr yr, P2 = sum xi yi,
// P3 = sum (xr + xi)(yr + yi)), so one complex multiply-add costs three
// DFMAs instead of four.  GB300 retires ~2 DFMA per clock per SM and no
// faster FP64 form exists on it (its FP64 tensor rate is the same), so the
// kernel is built to keep that pipe busy and nothing else: register tiles of
// 4 x 2 outputs per thread, operands staged through shared memory as three
// planes (re, im, re + im -- the sums formed once per staged element, not
// once per product), two blocks per SM so that one stages while the other
// computes.  Shared-memory and HBM traffic are a few percent of the DFMA
// time.  Each output sums its k range in increasing k in one thread, and
// split-k partials are added in split order: the results are bit-reproducible.
#include <algorithm>
#include <atomic>
#include <cstdio>

#include "gpp_gemm.h"
#include "gpp_gemm_mixed.h"
#include "gpp_ozaki.h"

namespace gpp {

gpp_status set_error(gpp_status s, const char *msg);

namespace {

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

gpp_status cuda_fail(cudaError_t e, const char *what) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return set_error(e == cudaErrorMemoryAllocation ? GPP_ERR_OUT_OF_MEMORY : GPP_ERR_CUDA, buf);
}

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// zgemm3m_kernel: Out[m][n] = sum_{k in split} X(m, k) Y(n, k), complex FP64.
// X(m, k) = X[m * xs + k] when XKFast, else X[k * xs + m]; Y likewise.  Block
// tile kBM x kBN outputs, kBK k values per shared-memory stage; thread
// (tx, ty) of a 16 x 16 grid owns rows ty + 16 i (i < kTM) and columns
// tx + 16 j (j < kTN), so its shared-memory reads are broadcasts or runs of
// consecutive words.  blockIdx.z is the k split: it covers
// [z * k_per_split, min(K, (z + 1) * k_per_split)) and writes its partial at
// Out + z * split_stride.
constexpr int kBM = 64, kBN = 32, kBK = 32, kTM = 4, kTN = 2, kGThreads = 256;
constexpr int kXP = kBM + 1, kYP = kBN + 1;  // padded plane rows
constexpr size_t kGemmSmem = sizeof(double) * 3 * kBK * (kXP + kYP);

template <bool XKFast, bool YKFast>
__global__ void __launch_bounds__(kGThreads, 2)
zgemm3m_kernel(const double2 *__restrict__ X, long long xs, const double2 *__restrict__ Y,
               long long ys, double2 *__restrict__ Out, long long out_ld, long long split_stride,
               int M, int N, int K, int k_per_split) {
    extern __shared__ double smem[];
    double *xr = smem, *xi = xr + kBK * kXP, *xsum = xi + kBK * kXP;
    double *yr = xsum + kBK * kXP, *yi = yr + kBK * kYP, *ysum = yi + kBK * kYP;
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    const int kb = blockIdx.z * k_per_split;
    const int ke = min(K, kb + k_per_split);
    double p1[kTM][kTN], p2[kTM][kTN], p3[kTM][kTN];
#pragma unroll
    for (int i = 0; i < kTM; ++i)
#pragma unroll
        for (int j = 0; j < kTN; ++j) p1[i][j] = p2[i][j] = p3[i][j] = 0.0;

    for (int k0 = kb; k0 < ke; k0 += kBK) {
        // Stage X (kBM x kBK) and Y (kBN x kBK) as re / im / re+im planes,
        // zero outside the matrix; reads are coalesced along the unit stride.
#pragma unroll 4
        for (int e = t; e < kBM * kBK; e += kGThreads) {
            const int k = XKFast ? e % kBK : e / kBM, m = XKFast ? e / kBK : e % kBM;
            double2 v = make_double2(0.0, 0.0);
            if (m0 + m < M && k0 + k < ke)
                v = __ldg(X + (XKFast ? (long long)(m0 + m) * xs + (k0 + k)
                                      : (long long)(k0 + k) * xs + (m0 + m)));
            xr[k * kXP + m] = v.x;
            xi[k * kXP + m] = v.y;
            xsum[k * kXP + m] = v.x + v.y;
        }
#pragma unroll 4
        for (int e = t; e < kBN * kBK; e += kGThreads) {
            const int k = YKFast ? e % kBK : e / kBN, n = YKFast ? e / kBK : e % kBN;
            double2 v = make_double2(0.0, 0.0);
            if (n0 + n < N && k0 + k < ke)
                v = __ldg(Y + (YKFast ? (long long)(n0 + n) * ys + (k0 + k)
                                      : (long long)(k0 + k) * ys + (n0 + n)));
            yr[k * kYP + n] = v.x;
            yi[k * kYP + n] = v.y;
            ysum[k * kYP + n] = v.x + v.y;
        }
        __syncthreads();
#pragma unroll 2
        for (int k = 0; k < kBK; ++k) {
            double ar[kTM], ai[kTM], as[kTM], br[kTN], bi[kTN], bs[kTN];
#pragma unroll
            for (int i = 0; i < kTM; ++i) {
                ar[i] = xr[k * kXP + ty + 16 * i];
                ai[i] = xi[k * kXP + ty + 16 * i];
                as[i] = xsum[k * kXP + ty + 16 * i];
            }
#pragma unroll
            for (int j = 0; j < kTN; ++j) {
                br[j] = yr[k * kYP + tx + 16 * j];
                bi[j] = yi[k * kYP + tx + 16 * j];
                bs[j] = ysum[k * kYP + tx + 16 * j];
            }
#pragma unroll
            for (int i = 0; i < kTM; ++i)
#pragma unroll
                for (int j = 0; j < kTN; ++j) {
                    p1[i][j] = fma(ar[i], br[j], p1[i][j]);
                    p2[i][j] = fma(ai[i], bi[j], p2[i][j]);
                    p3[i][j] = fma(as[i], bs[j], p3[i][j]);
                }
        }
        __syncthreads();
    }
    double2 *out = Out + (long long)blockIdx.z * split_stride;
#pragma unroll
    for (int i = 0; i < kTM; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < kTN; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n < N)
                out[(long long)m * out_ld + n] =
                    make_double2(p1[i][j] - p2[i][j], p3[i][j] - p1[i][j] - p2[i][j]);
        }
    }
}

// k values per split when a K-long sum is cut `splits` ways: split
// boundaries fall on kBK multiples, so every stage but a split's last is full.
int zgemm_k_per_split(int K, int splits) { return ceil_div(ceil_div(K, splits), kBK) * kBK; }
// Number of non-empty splits that makes (<= splits).
int zgemm_splits(int K, int splits) { return ceil_div(K, zgemm_k_per_split(K, splits)); }

// Launches zgemm3m_kernel over an M x N output with zgemm_splits(K, splits)
// k splits, split z written at Out + z * split_stride.
template <bool XKFast, bool YKFast>
cudaError_t launch_zgemm3m(const double2 *X, long long xs, const double2 *Y, long long ys,
                           double2 *Out, long long out_ld, long long split_stride, int M, int N,
                           int K, int splits, cudaStream_t s) {
    // The shared-memory opt-in is set once per device (host threads may race
    // to set it; setting it twice is harmless).
    static std::atomic<bool> configured[256] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (!configured[dev & 255].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(zgemm3m_kernel<XKFast, YKFast>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem);
        if (e != cudaSuccess) return e;
        configured[dev & 255].store(true, std::memory_order_release);
    }
    const int per = zgemm_k_per_split(K, splits);
    const int z = ceil_div(K, per);
    if (ceil_div(M, kBM) > 65535 || z > 65535)
        return cudaErrorInvalidConfiguration;
    dim3 grid((unsigned)ceil_div(N, kBN), (unsigned)ceil_div(M, kBM), (unsigned)z);
    zgemm3m_kernel<XKFast, YKFast><<<grid, kGThreads, kGemmSmem, s>>>(
        X, xs, Y, ys, Out, out_ld, split_stride, M, N, K, per);
    count_launch();
    return cudaGetLastError();
}

// k splits of the per-band GEMM (H = aqsn M_2^T sums over all ncouls
// columns): on the FP64 pipe enough blocks for ~10 waves of two blocks per
// SM; on the tensor cores (128 x 128 output tiles, so only 4 x 13 tiles at
// the production shape) 32 splits make ~5 waves.
constexpr int kHSplits = 8;
constexpr int kHSplitsTensor = 32;
int h_splits() { return fp64_gemm_on_tensor_cores() ? kHSplitsTensor : kHSplits; }

// c[k][r] for bands b0 + k (k < K) and rows [r0, r1); rows whose G' index
// is invalid get 0 (their fault bit is set, as in the per-term epilogue).
__global__ void __launch_bounds__(kThreads) gemm_coeff_kernel(Problem p, int b0, int K, int r0,
                                                              int r1, double2 *C, int *err) {
    const int nr = r1 - r0;
    const long long n = (long long)K * nr;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int k = (int)(i / nr), r = r0 + (int)(i % nr);
        const int igp = resolve_igp(p, r, err);
        double2 c = make_double2(0.0, 0.0);
        if (igp >= 0) {
            const double2 m = __ldg(p.aqsm + (size_t)(b0 + k) * p.nc + igp);
            c = cscale(make_double2(0.5 * m.x, -0.5 * m.y), __ldg(p.vcoul + igp));
        }
        C[(size_t)k * p.ng + r] = c;
    }
}

// One block per row tile (rows 2j, 2j+1): sum over ig of M_iw G for NWC
// frequencies from iw0, written as the row tile's block partial.
template <int NWC>
__global__ void __launch_bounds__(kThreads) gemm_epilogue_kernel(Problem p, Partials part,
                                                                 const double2 *G,
                                                                 int row_tile0) {
    constexpr int RG = 2, K = RG * NWC * 2;
    __shared__ double red[(kThreads / 32) * K];
    __shared__ double S[K];
    const int row_tile = row_tile0 + blockIdx.x;
    const int iw0 = blockIdx.y * NWC;
    const int nc = p.nc;
    double wx[NWC];
#pragma unroll
    for (int w = 0; w < NWC; ++w) wx[w] = __ldg(p.wx + min(iw0 + w, p.nw - 1));
    double2 acc[RG][NWC];
#pragma unroll
    for (int g = 0; g < RG; ++g)
#pragma unroll
        for (int w = 0; w < NWC; ++w) acc[g][w] = make_double2(0.0, 0.0);
#pragma unroll
    for (int g = 0; g < RG; ++g) {
        const int r = row_tile * RG + g;
        if (r >= p.ng) continue;
        const double2 *grow = G + (size_t)r * nc;
        const double2 *wrow = p.wt + (size_t)r * nc;
        const double2 *erow = p.ieps + (size_t)r * nc;
        for (int ig = threadIdx.x; ig < nc; ig += kThreads) {
            const double2 wt = __ldg(wrow + ig);
            const double2 A = cmul(__ldg(grow + ig), cmul(wt, __ldg(erow + ig)));
            const double ayw = A.y * wt.y, axw = A.x * wt.y, wti2 = wt.y * wt.y;
#pragma unroll
            for (int w = 0; w < NWC; ++w) {
                const double wr = wx[w] - wt.x;        // Re(wdiff); Im(wdiff) = -Im(wtilde)
                const double rr = rcp_fp64(fma(wr, wr, wti2));
                acc[g][w].x = fma(rr, fma(A.x, wr, -ayw), acc[g][w].x);
                acc[g][w].y = fma(rr, fma(A.y, wr, axw), acc[g][w].y);
            }
        }
    }
    double v[K];
#pragma unroll
    for (int g = 0; g < RG; ++g)
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            v[(g * NWC + w) * 2] = acc[g][w].x;
            v[(g * NWC + w) * 2 + 1] = acc[g][w].y;
        }
    block_reduce<K, kThreads>(v, red, S);
    const int w = threadIdx.x;
    if (w < NWC && iw0 + w < p.nw) {
        double2 tot = make_double2(0.0, 0.0);
#pragma unroll
        for (int g = 0; g < RG; ++g)
            tot = cadd(tot, make_double2(S[(g * NWC + w) * 2], S[(g * NWC + w) * 2 + 1]));
        part.ach[(long long)(iw0 + w) * part.ach_seg + part.ach_tile0 + row_tile] = tot;
    }
}

// M_2[r][ig] = Q conj(wdiff) / |wdiff|^2 at iw = 2, rows [r0, r1).
__global__ void __launch_bounds__(kThreads) gemm_m2_kernel(Problem p, int r0, int r1, double2 *M) {
    const size_t nc = (size_t)p.nc;
    const size_t n = (size_t)(r1 - r0) * nc;
    const double wx = __ldg(p.wx + 2);
    for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (size_t)gridDim.x * kThreads) {
        const size_t at = (size_t)r0 * nc + i;
        const double2 wt = __ldg(p.wt + at);
        const double2 Q = cmul(wt, __ldg(p.ieps + at));
        const double wr = wx - wt.x;
        const double rr = rcp_fp64(fma(wr, wr, wt.y * wt.y));
        M[at] = make_double2(rr * fma(Q.x, wr, -Q.y * wt.y), rr * fma(Q.y, wr, Q.x * wt.y));
    }
}

// acht_n1_loc partials: band b0 + k, row tile j: sum over the tile's rows of
// c[k][r] H[k][r], H being the sum of the per-band GEMM's k splits (added in
// split order).
__global__ void __launch_bounds__(kThreads) gemm_n1_kernel(Problem p, Partials part, int b0,
                                                           int K, int tile0, int tiles,
                                                           const double2 *C, const double2 *H,
                                                           int splits) {
    const long long n = (long long)K * tiles;
    const size_t split_stride = (size_t)K * p.ng;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int k = (int)(i / tiles), j = tile0 + (int)(i % tiles);
        double2 tot = make_double2(0.0, 0.0);
        for (int g = 0; g < 2; ++g) {
            const int r = 2 * j + g;
            if (r >= p.ng) continue;
            const size_t at = (size_t)k * p.ng + r;
            double2 h = H[at];
            for (int z = 1; z < splits; ++z) h = cadd(h, H[z * split_stride + at]);
            tot = cadd(tot, cmul(C[at], h));
        }
        part.n1[(long long)(b0 + k) * part.n1_seg + j] = tot;
    }
}

int grid_for(long long n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (n + kThreads - 1) / kThreads;
    const long long cap = (long long)(sms > 0 ? sms : 132) * 8;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

int nwc_of(int nw) { return nw <= 4 ? nw : 8; }

template <int NWC>
cudaError_t launch_epilogue_t(const Problem &p, const Partials &part, const double2 *G, RowTiles r,
                              cudaStream_t s) {
    dim3 grid((unsigned)(r.end - r.begin), (unsigned)ceil_div(p.nw, NWC));
    gemm_epilogue_kernel<NWC><<<grid, kThreads, 0, s>>>(p, part, G, r.begin);
    count_launch();
    return cudaGetLastError();
}


}  // namespace

// Scratch of the tensor-core GEMMs: G's, then (reused) H's.
size_t ozaki_scratch(const Problem &p, int bands, bool want_n1) {
    if (!fp64_gemm_on_tensor_cores()) return 0;
    size_t b = ozaki_bytes(p.ng, p.nc, bands, 1);
    if (want_n1) b = std::max(b, ozaki_bytes(bands, p.ng, p.nc, kHSplitsTensor));
    return b;
}

size_t gemm_bytes(const Problem &p, int bands, bool want_n1) {
    const size_t k = (size_t)bands, ng = (size_t)p.ng, nc = (size_t)p.nc;
    size_t b = align_up(sizeof(double2) * k * ng) + align_up(sizeof(double2) * ng * nc);
    if (want_n1)
        b += align_up(sizeof(double2) * ng * nc) + align_up(sizeof(double2) * h_splits() * k * ng);
    return b + align_up(ozaki_scratch(p, bands, want_n1));
}

namespace {

struct GemmBuffers {
    double2 *C, *G, *M2, *H;
    void *oz;  // tensor-core GEMM scratch
};

GemmBuffers carve(const Problem &p, void *ws, int K, bool want_n1) {
    const size_t ng = (size_t)p.ng, nc = (size_t)p.nc;
    char *w = static_cast<char *>(ws);
    GemmBuffers b{};
    b.C = reinterpret_cast<double2 *>(w);
    w += align_up(sizeof(double2) * (size_t)K * ng);
    b.G = reinterpret_cast<double2 *>(w);
    w += align_up(sizeof(double2) * ng * nc);
    if (want_n1) {
        b.M2 = reinterpret_cast<double2 *>(w);
        w += align_up(sizeof(double2) * ng * nc);
        b.H = reinterpret_cast<double2 *>(w);
        w += align_up(sizeof(double2) * h_splits() * (size_t)K * ng);
    }
    b.oz = w;
    return b;
}

}  // namespace

const double2 *gemm_g(const Problem &p, void *ws, int bands, bool want_n1) {
    return carve(p, ws, bands, want_n1).G;
}

gpp_status gemm_band_sum(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                         cudaStream_t s, cudaEvent_t after_slices) {
    const int K = b1 - b0;
    if (K <= 0 || p.ng <= 0) return GPP_OK;
    const GemmBuffers b = carve(p, ws, K, part.n1 != nullptr);
    gemm_coeff_kernel<<<grid_for((long long)K * p.ng), kThreads, 0, s>>>(p, b0, K, 0, p.ng, b.C,
                                                                         part.err);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gemm_coeff_kernel");
    // G (ng x nc) = C^T aqsn: X(r, k) = C[k][r], Y(ig, k) = aqsn[b0 + k][ig].
    if (fp64_gemm_on_tensor_cores()) {
        const OzOperand X{b.C, p.ng, false, p.ng}, Y{p.aqsn + (size_t)b0 * p.nc, p.nc, false, p.nc};
        e = ozaki_zgemm(X, Y, p.ng, p.nc, K, 1, b.G, p.nc, 0, b.oz, part.err, s, after_slices);
        if (e != cudaSuccess) return cuda_fail(e, "ozaki_zgemm (band sum)");
        return GPP_OK;
    }
    e = launch_zgemm3m<false, false>(b.C, p.ng, p.aqsn + (size_t)b0 * p.nc, p.nc, b.G, p.nc, 0,
                                     p.ng, p.nc, K, 1, s);
    if (e == cudaSuccess && after_slices) e = cudaEventRecord(after_slices, s);
    if (e != cudaSuccess) return cuda_fail(e, "zgemm3m_kernel (band sum)");
    return GPP_OK;
}

gpp_status gemm_rows(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                     cudaStream_t s, RowTiles rows) {
    const RowTiles rt = rows.clip(ceil_div(p.ng, 2));
    if (rt.end <= rt.begin || b1 <= b0) return GPP_OK;
    const GemmBuffers b = carve(p, ws, b1 - b0, part.n1 != nullptr);
    cudaError_t e;
    switch (nwc_of(p.nw)) {
        case 1: e = launch_epilogue_t<1>(p, part, b.G, rt, s); break;
        case 2: e = launch_epilogue_t<2>(p, part, b.G, rt, s); break;
        case 3: e = launch_epilogue_t<3>(p, part, b.G, rt, s); break;
        case 4: e = launch_epilogue_t<4>(p, part, b.G, rt, s); break;
        default: e = launch_epilogue_t<8>(p, part, b.G, rt, s); break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "gemm_epilogue_kernel");
    return GPP_OK;
}

gpp_status gemm_per_band(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                         cudaStream_t s, void *split_ws) {
    const int K = b1 - b0;
    if (K <= 0 || p.ng <= 0 || !part.n1) return GPP_OK;
    const GemmBuffers b = carve(p, ws, K, true);
    cudaError_t e = cudaSuccess;
    if (split_ws) {
        const gpp_status st = mixed_m2_fp64(p, split_ws, b0, b.M2, s);
        if (st != GPP_OK) return st;
    } else {
        gemm_m2_kernel<<<grid_for((long long)p.ng * p.nc), kThreads, 0, s>>>(p, 0, p.ng, b.M2);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "gemm_m2_kernel");
    }
    // H (K x ng) = aqsn M_2^T: X(k', ig) = aqsn[b0 + k'][ig], Y(r, ig) = M_2[r][ig],
    // the ncouls sum split up to h_splits() ways.
    int splits;
    if (fp64_gemm_on_tensor_cores()) {
        const OzOperand X{p.aqsn + (size_t)b0 * p.nc, p.nc, true, K}, Y{b.M2, p.nc, true, p.ng};
        e = ozaki_zgemm(X, Y, K, p.ng, p.nc, kHSplitsTensor, b.H, p.ng, (long long)K * p.ng, b.oz,
                        part.err, s);
        if (e != cudaSuccess) return cuda_fail(e, "ozaki_zgemm (per-band output)");
        splits = ozaki_splits(p.nc, kHSplitsTensor);
    } else {
        e = launch_zgemm3m<true, true>(p.aqsn + (size_t)b0 * p.nc, p.nc, b.M2, p.nc, b.H, p.ng,
                                       (long long)K * p.ng, K, p.ng, p.nc, kHSplits, s);
        if (e != cudaSuccess) return cuda_fail(e, "zgemm3m_kernel (per-band output)");
        splits = zgemm_splits(p.nc, kHSplits);
    }
    const int tiles = ceil_div(p.ng, 2);
    gemm_n1_kernel<<<grid_for((long long)K * tiles), kThreads, 0, s>>>(p, part, b0, K, 0, tiles,
                                                                       b.C, b.H, splits);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gemm_n1_kernel");
    return GPP_OK;
}

}  // namespace gpp

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
// G is one complex GEMM over the bands (cuBLAS cublasZgemm3m: the 3M form,
// three real FP64 GEMMs instead of four, 187 ms against 231 ms for
// cublasZgemm at the production shape on GB300; FP64 complex has no tcgen05
// form), and a fused pass over (r, ig) builds M on the fly and sums M G per
// row tile -- the same block-partial slots and fixed-order reduction as the
// per-term kernels.  The per-band output acht_n1_loc (iw = 2) needs
//   acht_n1_loc[n1] = sum_r c[n1][r] H[n1][r],  H[n1][r] = sum_ig aqsn[n1][ig] M_2[r][ig],
// a second GEMM against M_2 stored once.  Exact in real arithmetic; only
// the order of the FP64 roundings differs from the per-term kernel (and the
// 3M form's own, within ~1e-15 of the sums here).
#include <cublas_v2.h>

#include <algorithm>
#include <cstdio>

#include "gpp_gemm.h"

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

struct Handle {
    int dev = -1;
    cublasHandle_t h = nullptr;
};
thread_local Handle t_blas;

cublasStatus_t blas_handle(cudaStream_t s, cublasHandle_t *out) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (t_blas.dev != dev) {
        if (t_blas.h) cublasDestroy(t_blas.h);
        t_blas.h = nullptr;
        t_blas.dev = -1;
        cublasStatus_t st = cublasCreate(&t_blas.h);
        if (st != CUBLAS_STATUS_SUCCESS) return st;
        t_blas.dev = dev;
    }
    cublasStatus_t st = cublasSetStream(t_blas.h, s);
    *out = t_blas.h;
    return st;
}

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
// c[k][r] H[k][r].
__global__ void __launch_bounds__(kThreads) gemm_n1_kernel(Problem p, Partials part, int b0,
                                                           int K, int tile0, int tiles,
                                                           const double2 *C, const double2 *H) {
    const long long n = (long long)K * tiles;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int k = (int)(i / tiles), j = tile0 + (int)(i % tiles);
        double2 tot = make_double2(0.0, 0.0);
        for (int g = 0; g < 2; ++g) {
            const int r = 2 * j + g;
            if (r >= p.ng) continue;
            const size_t at = (size_t)k * p.ng + r;
            tot = cadd(tot, cmul(C[at], H[at]));
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

gpp_status blas_fail(cublasStatus_t st, const char *what) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s failed (cuBLAS status %d)", what, (int)st);
    return set_error(st == CUBLAS_STATUS_ALLOC_FAILED ? GPP_ERR_OUT_OF_MEMORY : GPP_ERR_CUDA, buf);
}

}  // namespace

size_t gemm_bytes(const Problem &p, int bands, bool want_n1) {
    const size_t k = (size_t)bands, ng = (size_t)p.ng, nc = (size_t)p.nc;
    size_t b = align_up(sizeof(double2) * k * ng) + align_up(sizeof(double2) * ng * nc);
    if (want_n1) b += align_up(sizeof(double2) * ng * nc) + align_up(sizeof(double2) * k * ng);
    return b;
}

namespace {

struct GemmBuffers {
    double2 *C, *G, *M2, *H;
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
    }
    return b;
}

const cuDoubleComplex kOne = {1.0, 0.0}, kZero = {0.0, 0.0};

}  // namespace

gpp_status gemm_band_sum(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                         cudaStream_t s) {
    const int K = b1 - b0;
    if (K <= 0 || p.ng <= 0) return GPP_OK;
    const GemmBuffers b = carve(p, ws, K, part.n1 != nullptr);
    gemm_coeff_kernel<<<grid_for((long long)K * p.ng), kThreads, 0, s>>>(p, b0, K, 0, p.ng, b.C,
                                                                         part.err);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gemm_coeff_kernel");
    cublasHandle_t h = nullptr;
    cublasStatus_t bs = blas_handle(s, &h);
    if (bs != CUBLAS_STATUS_SUCCESS) return blas_fail(bs, "cublasCreate/cublasSetStream");
    // Column-major view: aqsn rows are columns of an (nc x K) matrix, C of an
    // (ng x K) one, G of an (nc x ng) one: G = aqsn * C^T.
    bs = cublasZgemm3m(h, CUBLAS_OP_N, CUBLAS_OP_T, p.nc, p.ng, K, &kOne,
                     reinterpret_cast<const cuDoubleComplex *>(p.aqsn + (size_t)b0 * p.nc), p.nc,
                     reinterpret_cast<const cuDoubleComplex *>(b.C), p.ng, &kZero,
                     reinterpret_cast<cuDoubleComplex *>(b.G), p.nc);
    if (bs != CUBLAS_STATUS_SUCCESS) return blas_fail(bs, "cublasZgemm (band sum)");
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
                         cudaStream_t s) {
    const int K = b1 - b0;
    if (K <= 0 || p.ng <= 0 || !part.n1) return GPP_OK;
    const GemmBuffers b = carve(p, ws, K, true);
    gemm_m2_kernel<<<grid_for((long long)p.ng * p.nc), kThreads, 0, s>>>(p, 0, p.ng, b.M2);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gemm_m2_kernel");
    cublasHandle_t h = nullptr;
    cublasStatus_t bs = blas_handle(s, &h);
    if (bs != CUBLAS_STATUS_SUCCESS) return blas_fail(bs, "cublasCreate/cublasSetStream");
    // H (column-major ng x K) = M_2^T * aqsn.
    bs = cublasZgemm3m(h, CUBLAS_OP_T, CUBLAS_OP_N, p.ng, K, p.nc, &kOne,
                     reinterpret_cast<const cuDoubleComplex *>(b.M2), p.nc,
                     reinterpret_cast<const cuDoubleComplex *>(p.aqsn + (size_t)b0 * p.nc), p.nc,
                     &kZero, reinterpret_cast<cuDoubleComplex *>(b.H), p.ng);
    if (bs != CUBLAS_STATUS_SUCCESS) return blas_fail(bs, "cublasZgemm (per-band output)");
    const int tiles = ceil_div(p.ng, 2);
    gemm_n1_kernel<<<grid_for((long long)K * tiles), kThreads, 0, s>>>(p, part, b0, K, 0, tiles,
                                                                       b.C, b.H);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gemm_n1_kernel");
    return GPP_OK;
}

}  // namespace gpp

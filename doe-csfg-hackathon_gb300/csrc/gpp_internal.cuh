// gpp_internal.cuh -- shared device-side definitions of the GB300 GPP sigma
// kernels (FP64, mixed precision, batched) and the host dispatcher.
//
// Data layout in HBM (caller-owned, unchanged from the reference,
// gppKerSeq.cpp:194-197): complex128 arrays interleaved {re,im}, row-major;
// aqsntemp/aqsmtemp [number_bands][ncouls], I_eps/wtilde [ngpown][ncouls].
// Library scratch (per-device workspace): per-block partial sums (complex128)
// reduced in a fixed order by gpp_reduce_kernel, and for the mixed path the
// float-float split copies of the inputs made by the prep kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gpp {

// Constants of ssxt_scht_solver (gppComplex_seq.cpp:20-23) and of the main
// drivers (gppComplex_seq.cpp:241-247).
constexpr double kTo1 = 1e-6;
constexpr double kSexcut = 4.0;
constexpr double kLimitOne = 1.0 / (kTo1 * 4.0);
constexpr double kLimitTwo = 0.25;  // pow(0.5, 2)

enum : int { kSemComplexSeq = 0, kSemKerSeq = 1 };

// Device-side fault bits (workspace word, read by gpp_wait).
enum : int { kErrBadIgp = 1, kErrBadIndinv = 2, kErrPipelineTimeout = 4 };

// Iteration cap of every device-side wait (mbarrier polls): a wait that runs
// out raises kErrPipelineTimeout and the block abandons its tile.
constexpr int kWaitLimit = 1 << 22;

// Everything a sigma kernel needs about one problem (one quasiparticle
// state).  Passed by value as a kernel parameter or read from a table by the
// batched kernel.
struct Problem {
    const double2 *aqsm;   // [nb][nc]
    const double2 *aqsn;   // [nb][nc]
    const double2 *ieps;   // [ng][nc]
    const double2 *wt;     // [ng][nc]
    const double *vcoul;   // [nc]
    const int *inv_igp;    // [ng]
    const int *indinv;     // [nc] or null
    const double *wx;      // wx(n1, iw) = wx[n1 * wx_stride + iw]
    int wx_stride;
    int nb, nv, nc, ng, nw;
    double occ;
    int semantics;
};

// Where one launch writes its per-block partial sums.  Segment layouts:
//   ach[iw * ach_seg + tile]   (ach_seg = tiles of all launches of the call)
//   asx[iw * asx_seg + tile]   (occupied-band launches only)
//   n1[band * n1_seg + row_tile] (acht_n1_loc, only when nw >= 3)
struct Partials {
    double2 *ach;
    long long ach_seg;
    int ach_tile0;   // first tile index of this launch inside the ach segment
    double2 *asx;
    long long asx_seg;
    double2 *n1;     // may be null
    int n1_seg;
    int *err;        // device fault word
};

// Resolve the G' column index of local row my_igp exactly like the reference
// (gppComplex_seq.cpp:342-344: values >= ncouls clamp to ncouls-1), then the
// optional indinv remap.  Returns -1 (and raises a fault bit) for indices the
// reference would read out of bounds.
__device__ __forceinline__ int resolve_igp(const Problem &p, int my_igp, int *err) {
    int igp = __ldg(p.inv_igp + my_igp);
    if (igp >= p.nc) igp = p.nc - 1;
    if (igp < 0) {
        atomicOr(err, kErrBadIgp);
        return -1;
    }
    if (p.indinv) {
        igp = __ldg(p.indinv + igp);
        if (igp < 0 || igp >= p.nc) {
            atomicOr(err, kErrBadIndinv);
            return -1;
        }
    }
    return igp;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmul_conj_b(double2 a, double2 b) {  // a * conj(b)
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
    return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 cscale(double2 a, double s) {
    return make_double2(a.x * s, a.y * s);
}

// The same complex operations with every rounding written out: __fma_rn,
// __dmul_rn and __dadd_rn are never contracted or reassociated, so code built
// from them gives the same bits in every kernel that inlines it, whatever
// the compiler would fuse around a plain a*b + c in each instantiation.
__device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
    return make_double2(__fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y)),
                        __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 cmul_conj_b_rn(double2 a, double2 b) {  // a * conj(b)
    return make_double2(__fma_rn(a.x, b.x, __dmul_rn(a.y, b.y)),
                        __fma_rn(a.y, b.x, -__dmul_rn(a.x, b.y)));
}
__device__ __forceinline__ double2 cscale_rn(double2 a, double s) {
    return make_double2(__dmul_rn(a.x, s), __dmul_rn(a.y, s));
}
__device__ __forceinline__ double abs2_rn(double2 a) {
    return __fma_rn(a.x, a.x, __dmul_rn(a.y, a.y));
}
// acc + a*b in two FMAs per component.
__device__ __forceinline__ double2 cmul_acc_rn(double2 acc, double2 a, double2 b) {
    return make_double2(__fma_rn(a.x, b.x, __fma_rn(-a.y, b.y, acc.x)),
                        __fma_rn(a.x, b.y, __fma_rn(a.y, b.x, acc.y)));
}

// FP64 reciprocal: hardware seed (rcp.approx.ftz.f64, issued to the
// multi-function unit, not the FP64 pipe) refined by one cubic Newton-Raphson
// step r = r0 (1 + e + e^2), e = 1 - d r0 (the classical Newton iteration for
// 1/d with the second-order term kept).  Three FP64 FMAs instead of the ~5
// FMA-equivalents of an IEEE division; the error is within about one ulp.
__device__ __forceinline__ double rcp_fp64(double d) {
    double r0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(d));
    double e = fma(-d, r0, 1.0);
    double t = fma(e, e, e);
    return fma(r0, t, r0);
}

// Warp-level sum of a double with a fixed shuffle tree (deterministic).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

// Block-wide reduction of K doubles per thread (fixed shuffle tree within a
// warp, fixed warp order across warps); the sums land in out[K] (shared).
template <int K, int THREADS>
__device__ __forceinline__ void block_reduce(double (&v)[K], double *red, double *out) {
    constexpr int NWARP = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = warp_sum(v[k]);
        if (lane == 0) red[warp * K + k] = s;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += THREADS) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < NWARP; ++w) s += red[w * K + k];
        out[k] = s;
    }
    __syncthreads();
}

// Epilogue of an unoccupied-band block: S holds, per (band n, row g,
// frequency w), the ig sum of aqsn * Q * conj(wdiff) / |wdiff|^2 as
// S[((n*RG + g)*NWC + w)*2 + {0,1}].  Weight each (n1, igp) sum by
// 0.5 vcoul[igp] conj(aqsm[n1,igp]) (gppComplex_seq.cpp:146,374,379), add
// the pairs in a fixed order and store one partial per frequency (threads
// 0..NWC-1) and, for the iw = 2 column, one per band (threads 32..32+RN-1).
template <int RN, int RG, int NWC>
__device__ __forceinline__ void noflag_epilogue(const Problem &p, const Partials &part,
                                                const double *S, int row0, int band0,
                                                int band_end, int iw0, long long tile_in_launch,
                                                int row_tile) {
    const long long tile = tile_in_launch + part.ach_tile0;
    const int t = threadIdx.x;
    if (!(t < NWC || (part.n1 && t >= 32 && t < 32 + RN))) return;
    const bool is_n1 = t >= 32;
    const int nlo = is_n1 ? t - 32 : 0, nhi = is_n1 ? t - 32 + 1 : RN;
    const int w = is_n1 ? 2 - iw0 : t;
    if (w < 0 || w >= NWC || iw0 + w >= p.nw) return;
    double2 tot = make_double2(0.0, 0.0);
    for (int n = nlo; n < nhi; ++n) {
        const int b = band0 + n;
        if (b >= band_end) continue;
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            const int row = row0 + g;
            if (row >= p.ng) continue;
            const int igp = resolve_igp(p, row, part.err);
            if (igp < 0) continue;
            const double2 m = __ldg(p.aqsm + (size_t)b * p.nc + igp);
            const int k = ((n * RG + g) * NWC + w) * 2;
            const double2 s = cmul(make_double2(m.x, -m.y), make_double2(S[k], S[k + 1]));
            tot = cadd(tot, cscale(cscale(s, 0.5), __ldg(p.vcoul + igp)));
        }
    }
    if (!is_n1)
        part.ach[(long long)(iw0 + w) * part.ach_seg + tile] = tot;
    else if (band0 + nlo < band_end)
        part.n1[(long long)(band0 + nlo) * part.n1_seg + row_tile] = tot;
}

}  // namespace gpp

// gpp_ozaki.cu -- FP64-class complex GEMM on the tensor cores.
//
// GB300 retires about 1.9 FP64 FMAs per clock per SM, so the band-sum GEMM
// of the FP64 path (gpp_gemm.cu) is bound by the FP64 pipe.  Its tensor
// cores are two orders of magnitude faster, and they can be made to compute
// FP64-accurate products by the splitting of Ozaki, Ogita, Oishi and Rump
// ("Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer.
// Algorithms 59, 2012):
//
//  * every real operand value x of row (or column) l and k chunk c is
//    written as x = 2^e sum_{i=1..S} s_i 2^(-7 i), e the chunk's common
//    exponent (max |x| < 2^e), s_1 in [-128, 128] and s_i in [-64, 64]:
//    integers, held exactly in bf16 (8 significant bits).  S = 8 slices keep
//    56 bits of the chunk's largest value;
//  * a product of two slices summed over a chunk of at most 512 k values is
//    an integer below 2^24 in magnitude, which the tensor cores' FP32
//    accumulation adds exactly (checked on the GB300 for sums up to 2^24
//    with operands up to 128);
//  * pairs (i, j) with the same i + j = d share the scale 2^(-7 d); those
//    whose worst-case sums still fit in 2^24 are summed in one accumulator
//    (10 groups for the 36 pairs with i + j <= 9), each group's exact
//    integer sum is stored, and a combining pass scales the group sums and
//    adds them in float-float;
//  * pairs with i + j > 9 fall below 2^-56 of the largest products and are
//    left out, as are bits past the 8th slice.
//
// Complex products take the 3M form (Gauss: re = P1 - P2, im = P3 - P1 -
// P2 with P1 = sum xr yr, P2 = sum xi yi, P3 = sum (xr + xi)(yr + yi)), so
// three real splittings and three real products, as in zgemm3m_kernel; the
// result agrees with that FP64 GEMM to about 1e-15 of its values.
//
// The tensor-core kernel uses warp-level mma.sync m16n8k16 (bf16 in, FP32
// accumulate): a block of 4 warps computes 128 x 128 outputs (64 x 64 per
// warp), staging 32 k of one slice pair per step through a four-stage
// cp.async ring in shared memory (rows padded to 80 bytes so ldmatrix is
// conflict-free), two blocks per SM.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "gpp_kernels.h"
#include "gpp_ozaki.h"
#include "gpp_ozaki_split.cuh"

namespace gpp {

namespace {

constexpr int kS = kOzSlices;    // slices per operand value
constexpr int kKcMax = 512;      // k values per chunk (exactness bound)
constexpr int kBM = 128, kBN = 128, kBK = 32;
constexpr int kThreads = 128;    // 4 warps: 2 along M x 2 along N, 64 x 64 each
constexpr int kLdk = kBK + 8;    // padded shared-memory row (80 bytes)
constexpr int kStages = 4;
constexpr size_t kGemmSmem = sizeof(__nv_bfloat16) * kStages * (kBM + kBN) * kLdk;  // 80 KB
constexpr int kGroups = 10;      // fold groups per (plane, chunk)

// The 36 slice pairs (i, j), i + j <= 9, in group order; kGroupEnd marks the
// last pair of each group (the fold point, scale 2^(-7 (i + j))).  Group
// worst cases (|s_1| <= 2^7, |s_i| <= 2^6, 512 k values): d = 2..7 whole
// (2^14 .. 2^15 per k); d = 8 and 9 in two groups each.
constexpr int kPairs = 36;
__constant__ unsigned char kPairI[kPairs] = {1, 1, 2, 1, 2, 3, 1, 2, 3, 4, 1, 2, 3, 4, 5, 1, 2, 3,
                                             4, 5, 6, 1, 2, 3, 4, 5, 6, 7, 1, 2, 3, 4, 5, 6, 7, 8};
__constant__ unsigned char kPairJ[kPairs] = {1, 2, 1, 3, 2, 1, 4, 3, 2, 1, 5, 4, 3, 2, 1, 6, 5, 4,
                                             3, 2, 1, 7, 6, 5, 4, 3, 2, 1, 8, 7, 6, 5, 4, 3, 2, 1};
__constant__ unsigned char kGroupEnd[kPairs] = {1, 0, 1, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0,
                                                0, 0, 1, 0, 0, 0, 0, 1, 0, 1, 0, 0, 0, 0, 1, 0, 0, 1};
// i + j of each group.
__constant__ unsigned char kGroupD[kGroups] = {2, 3, 4, 5, 6, 7, 8, 8, 9, 9};

struct Geometry {
    int M, N, K;       // logical sizes
    int Mp, Np;        // padded to the block tile
    int nch, Kc, Kp;   // chunks, chunk length (multiple of kBK), padded K = nch * Kc
    int cps, splits;   // chunks per split, splits
};

Geometry geometry(int M, int N, int K, int splits) {
    Geometry g;
    g.M = M;
    g.N = N;
    g.K = K;
    g.Mp = ceil_div(std::max(M, 1), kBM) * kBM;
    g.Np = ceil_div(std::max(N, 1), kBN) * kBN;
    g.nch = std::max(1, ceil_div(K, kKcMax));
    g.Kc = ceil_div(ceil_div(std::max(K, 1), g.nch), kBK) * kBK;
    g.Kp = g.nch * g.Kc;
    g.cps = ceil_div(g.nch, std::max(1, splits));
    g.splits = ceil_div(g.nch, g.cps);
    return g;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

struct Buffers {
    __nv_bfloat16 *sx, *sy;
    int *ex, *ey, *exmax, *eymax;
    float *fold;  // [splits][3][cps][kGroups][Mp][Np]: each group's exact integer sum
};

size_t fold_elems(const Geometry &g) {
    return (size_t)g.splits * 3 * g.cps * kGroups * g.Mp * g.Np;
}

Buffers carve(const Geometry &g, void *ws) {
    char *w = static_cast<char *>(ws);
    Buffers b;
    b.sx = reinterpret_cast<__nv_bfloat16 *>(w);
    w += align_up(sizeof(__nv_bfloat16) * 3 * kS * (size_t)g.Mp * g.Kp);
    b.sy = reinterpret_cast<__nv_bfloat16 *>(w);
    w += align_up(sizeof(__nv_bfloat16) * 3 * kS * (size_t)g.Np * g.Kp);
    b.ex = reinterpret_cast<int *>(w);
    w += align_up(sizeof(int) * (size_t)g.nch * g.Mp);
    b.ey = reinterpret_cast<int *>(w);
    w += align_up(sizeof(int) * (size_t)g.nch * g.Np);
    b.exmax = reinterpret_cast<int *>(w);
    w += align_up(sizeof(int) * (size_t)g.Mp);
    b.eymax = reinterpret_cast<int *>(w);
    w += align_up(sizeof(int) * (size_t)g.Np);
    b.fold = reinterpret_cast<float *>(w);
    return b;
}

__device__ __forceinline__ double2 operand_at(const OzOperand &z, int l, int k) {
    return __ldg(z.kfast ? z.z + (size_t)l * z.ld + k : z.z + (size_t)k * z.ld + l);
}

// Exponent of an all-zero chunk: far enough below any double's that every
// scale formed from it underflows to zero.
constexpr int kZeroExp = -4000;

// |x| as its bit pattern (monotone in |x| for every double but NaN).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned long long max3_bits(double2 v) {
    return max(max(abs_bits(v.x), abs_bits(v.y)), abs_bits(v.x + v.y));
}
// The e of frexp for the nonzero magnitude with bits b (b < 2^e).
__device__ __forceinline__ int exp_of_bits(unsigned long long b) {
    if (b == 0) return kZeroExp;
    const int E = (int)(b >> 52);
    return E > 0 ? E - 1022 : (63 - __clzll((long long)b)) - 1073;
}

// Largest |re|, |im|, |re + im| of Z(l, k) over chunk c, as an exponent e
// with max < 2^e (kZeroExp when the chunk is all zero), for l < Lp (rows
// past L are zero); compared as bit patterns on the integer pipes.  kfast: a
// warp per (l, c), lanes along k; else a block per (c, 32 consecutive l):
// lanes along l, the 8 warps interleaved along k, reduced through shared
// memory.
__global__ void __launch_bounds__(256) oz_exp_kernel(OzOperand z, int K, int Kc, int nch, int Lp,
                                                     int *E) {
    const long long n = (long long)nch * Lp;
    if (z.kfast) {
        const int lane = threadIdx.x & 31;
        for (long long w = ((long long)blockIdx.x * 256 + threadIdx.x) >> 5; w < n;
             w += ((long long)gridDim.x * 256) >> 5) {
            const int c = (int)(w / Lp), l = (int)(w % Lp);
            unsigned long long mx = 0;
            if (l < z.L)
                for (int k = c * Kc + lane; k < min(K, (c + 1) * Kc); k += 32)
                    mx = max(mx, max3_bits(operand_at(z, l, k)));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) E[w] = exp_of_bits(mx);
        }
    } else {
        __shared__ unsigned long long red[8][32];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int tiles = Lp / 32;  // Lp is a multiple of the block tile
        for (int b = blockIdx.x; b < nch * tiles; b += gridDim.x) {
            const int c = b / tiles, l = (b % tiles) * 32 + lane;
            unsigned long long mx = 0;
            if (l < z.L)
                for (int k = c * Kc + warp; k < min(K, (c + 1) * Kc); k += 8)
                    mx = max(mx, max3_bits(operand_at(z, l, k)));
            red[warp][lane] = mx;
            __syncthreads();
            if (warp == 0) {
#pragma unroll
                for (int w = 1; w < 8; ++w) mx = max(mx, red[w][lane]);
                E[(size_t)c * Lp + l] = exp_of_bits(mx);
            }
            __syncthreads();
        }
    }
}

// Emax[l] = max over chunks of E[c][l].
__global__ void __launch_bounds__(256) oz_emax_kernel(const int *E, int nch, int Lp, int *Emax) {
    for (int l = blockIdx.x * 256 + threadIdx.x; l < Lp; l += gridDim.x * 256) {
        int e = E[l];
        for (int c = 1; c < nch; ++c) e = max(e, E[(size_t)c * Lp + l]);
        Emax[l] = e;
    }
}

// Slices of the three real planes (re, im, re + im): out[((g S + i) Lp + l)
// Kp + k] = s_(i+1) of plane g at (l, k); zero outside L x K.  The slices
// are the balanced base-128 digits of round(x 2^(7 S - e)): s_2..s_S in
// [-64, 63], s_1 the rest (|s_1| <= 128), so x = 2^e sum_i s_i 2^(-7 i) to
// within 2^(e - 57).  Integer arithmetic throughout (the FP64 pipe is slow on
// GB300).  A thread per (l, k), k fastest.
__global__ void __launch_bounds__(256) oz_split_kernel(OzOperand z, int K, int Kc, int Kp, int Lp,
                                                       const int *E, __nv_bfloat16 *out) {
    const long long n = (long long)Lp * Kp;
    const size_t plane = (size_t)Lp * Kp;
    for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < n;
         t += (long long)gridDim.x * 256) {
        const int l = (int)(t / Kp), k = (int)(t % Kp);
        double2 v = make_double2(0.0, 0.0);
        if (l < z.L && k < K) v = operand_at(z, l, k);
        const int e = E[(size_t)(k / Kc) * Lp + l];
        const double r[3] = {v.x, v.y, v.x + v.y};
#pragma unroll
        for (int g = 0; g < 3; ++g) {
            int d[kS];
            oz_slices(r[g], e, d);
#pragma unroll
            for (int i = 0; i < kS; ++i)
                out[(size_t)(g * kS + i) * plane + t] = __int2bfloat16_rn(d[i]);
        }
    }
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void ldmatrix_x4(unsigned (&r)[4], const void *p) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(p));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// 2^e as a float for e >= -126 (exact), 0 below (a group that far below the
// largest products is under the float-float resolution).
__device__ __forceinline__ float pow2f(int e) {
    return e < -126 ? 0.0f : __int_as_float((e + 127) << 23);
}

// (h, l) += v in float-float (TwoSum, Knuth); v is exact.
__device__ __forceinline__ void df_acc(float &h, float &l, float v) {
    const float s = __fadd_rn(h, v);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    l = __fadd_rn(l, e);
    h = s;
}

// Position in a block's sequence of 32-k steps: plane g, chunk cl of the
// split, slice pair p, k step ks (fastest).
struct Step {
    int ks, p, cl, g;
    __device__ __forceinline__ void next(int KS, int nch_here) {
        if (++ks < KS) return;
        ks = 0;
        if (++p < kPairs) return;
        p = 0;
        if (++cl < nch_here) return;
        cl = 0;
        ++g;
    }
};

// The tensor-core products: block (bx, by) of split z runs, for each real
// plane g, chunk and slice pair, the 128 x 128 x 32 steps of the pair's
// product, and stores each group's exact FP32 sum at
// fold[((((z 3 + g) cps + cl) kGroups + group) Mp + m) Np + n].
__global__ void __launch_bounds__(kThreads, 2)
oz_gemm_kernel(const __nv_bfloat16 *__restrict__ SX, const __nv_bfloat16 *__restrict__ SY,
               int Mp, int Np, int Kp, int Kc, int cps, int nch, float *__restrict__ fold) {
    extern __shared__ __align__(128) __nv_bfloat16 smem[];
    __nv_bfloat16 (*sA)[kBM][kLdk] = reinterpret_cast<__nv_bfloat16 (*)[kBM][kLdk]>(smem);
    __nv_bfloat16 (*sB)[kBN][kLdk] =
        reinterpret_cast<__nv_bfloat16 (*)[kBN][kLdk]>(smem + (size_t)kStages * kBM * kLdk);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN, z = blockIdx.z;
    const int c0 = z * cps, nch_here = min(cps, nch - c0);
    const int KS = Kc / kBK;
    const long long T = 3LL * nch_here * kPairs * KS;
    const size_t xplane = (size_t)Mp * Kp, yplane = (size_t)Np * Kp, fplane = (size_t)Mp * Np;

    Step ahead{0, 0, 0, 0};  // the next step to stage
    auto issue = [&](int buf) {
        const Step &q = ahead;
        const size_t kof = (size_t)(c0 + q.cl) * Kc + (size_t)q.ks * kBK;
        const __nv_bfloat16 *a =
            SX + (size_t)(q.g * kS + kPairI[q.p] - 1) * xplane + (size_t)m0 * Kp + kof;
        const __nv_bfloat16 *b =
            SY + (size_t)(q.g * kS + kPairJ[q.p] - 1) * yplane + (size_t)n0 * Kp + kof;
#pragma unroll
        for (int r = 0; r < 8; ++r) {  // 1024 16-byte pieces, 4 per 32-k row
            const int piece = tid + r * kThreads;
            const int row = (piece >> 2) & (kBM - 1), part16 = piece & 3;
            if (piece < kBM * 4)
                cp_async16(&sA[buf][row][part16 * 8], a + (size_t)row * Kp + part16 * 8);
            else
                cp_async16(&sB[buf][row][part16 * 8], b + (size_t)row * Kp + part16 * 8);
        }
        ahead.next(KS, nch_here);
    };

    float acc[4][8][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

#pragma unroll
    for (int st = 0; st < kStages - 1; ++st) {
        if (st < T) issue(st);
        cp_async_commit();
    }
    Step cur{0, 0, 0, 0};
    int group = 0;
    for (long long t = 0; t < T; ++t) {
        cp_async_wait<kStages - 2>();
        __syncthreads();  // step t has landed; every warp is done with step t - 1
        if (t + kStages - 1 < T) issue((int)((t + kStages - 1) % kStages));
        cp_async_commit();
        const int buf = (int)(t % kStages);
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 16) {
            unsigned af[4][4], bfr[4][4];
#pragma unroll
            for (int mt = 0; mt < 4; ++mt)
                ldmatrix_x4(af[mt], &sA[buf][wm * 64 + mt * 16 + (lane & 15)][kk + (lane >> 4) * 8]);
#pragma unroll
            for (int np = 0; np < 4; ++np)
                ldmatrix_x4(bfr[np], &sB[buf][wn * 64 + np * 16 + (lane & 7) + ((lane >> 4) << 3)]
                                        [kk + ((lane >> 3) & 1) * 8]);
#pragma unroll
            for (int mt = 0; mt < 4; ++mt)
#pragma unroll
                for (int nt = 0; nt < 8; ++nt)
                    mma_bf16(acc[mt][nt], af[mt], bfr[nt >> 1][(nt & 1) * 2],
                             bfr[nt >> 1][(nt & 1) * 2 + 1]);
        }
        if (cur.ks == KS - 1 && kGroupEnd[cur.p]) {  // store the group's exact sums
            float *f = fold + ((((size_t)z * 3 + cur.g) * cps + cur.cl) * kGroups + group) * fplane;
#pragma unroll
            for (int mt = 0; mt < 4; ++mt)
#pragma unroll
                for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int m = m0 + wm * 64 + mt * 16 + (lane >> 2) + h * 8;
                        const int n = n0 + wn * 64 + nt * 8 + (lane & 3) * 2;
                        *reinterpret_cast<float2 *>(f + (size_t)m * Np + n) =
                            make_float2(acc[mt][nt][h * 2], acc[mt][nt][h * 2 + 1]);
                        acc[mt][nt][h * 2] = acc[mt][nt][h * 2 + 1] = 0.f;
                    }
            group = group + 1 == kGroups ? 0 : group + 1;
        }
        cur.next(KS, nch_here);
    }
}

// Out = (P1 - P2, P3 - P1 - P2) 2^(Emax_x[m] + Emax_y[n]) per split: each
// plane's group sums scaled by 2^(e_x - Emax_x + e_y - Emax_y - 7 d) for
// their chunk and added in float-float, in a fixed order; the three planes
// combined in FP64.
__global__ void __launch_bounds__(256) oz_combine_kernel(const float *fold, const int *EX,
                                                         const int *EY, const int *EXmax,
                                                         const int *EYmax, int M, int N, int Mp,
                                                         int Np, int cps, int nch, int splits,
                                                         double2 *Out, long long out_ld,
                                                         long long split_stride) {
    const long long n = (long long)splits * M * N;
    const size_t fplane = (size_t)Mp * Np;
    for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < n;
         t += (long long)gridDim.x * 256) {
        const int col = (int)(t % N);
        const long long q = t / N;
        const int row = (int)(q % M), z = (int)(q / M);
        const int c0 = z * cps, nch_here = min(cps, nch - c0);
        const int exm = __ldg(EXmax + row), eyn = __ldg(EYmax + col);
        double P[3];
        for (int g = 0; g < 3; ++g) {
            float h = 0.f, l = 0.f;
            for (int cl = 0; cl < nch_here; ++cl) {
                const int c = c0 + cl;
                const int sh = __ldg(EX + (size_t)c * Mp + row) - exm +
                               __ldg(EY + (size_t)c * Np + col) - eyn;
                const float *f = fold + ((((size_t)z * 3 + g) * cps + cl) * kGroups) * fplane +
                                 (size_t)row * Np + col;
#pragma unroll
                for (int grp = 0; grp < kGroups; ++grp)
                    df_acc(h, l, __ldg(f + grp * fplane) * pow2f(sh - 7 * kGroupD[grp]));
            }
            P[g] = (double)h + (double)l;
        }
        const int e = exm + eyn;
        Out[z * split_stride + (long long)row * out_ld + col] =
            make_double2(scalbn(P[0] - P[1], e), scalbn(P[2] - P[0] - P[1], e));
    }
}

int grid_for(long long n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (n + 255) / 256;
    const long long cap = (long long)(sms > 0 ? sms : 132) * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

size_t ozaki_bytes(int M, int N, int K, int splits) {
    const Geometry g = geometry(M, N, K, splits);
    return align_up(sizeof(__nv_bfloat16) * 3 * kS * (size_t)g.Mp * g.Kp) +
           align_up(sizeof(__nv_bfloat16) * 3 * kS * (size_t)g.Np * g.Kp) +
           align_up(sizeof(int) * (size_t)g.nch * g.Mp) + align_up(sizeof(int) * (size_t)g.nch * g.Np) +
           align_up(sizeof(int) * (size_t)g.Mp) + align_up(sizeof(int) * (size_t)g.Np) +
           align_up(sizeof(float) * fold_elems(g));
}

int ozaki_splits(int K, int splits) { return geometry(1, 1, K, splits).splits; }

cudaError_t ozaki_zgemm(const OzOperand &X, const OzOperand &Y, int M, int N, int K, int splits,
                        double2 *Out, long long out_ld, long long split_stride, void *ws,
                        cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    const Geometry g = geometry(M, N, K, splits);
    if (g.Mp / kBM > 65535 || g.Np / kBN > 65535 || g.splits > 65535)
        return cudaErrorInvalidConfiguration;
    const Buffers b = carve(g, ws);
    // kfast: a warp per (row, chunk); else a block per (chunk, 32 rows).
    oz_exp_kernel<<<grid_for((long long)g.nch * g.Mp * (X.kfast ? 32 : 8)), 256, 0, s>>>(
        X, K, g.Kc, g.nch, g.Mp, b.ex);
    oz_exp_kernel<<<grid_for((long long)g.nch * g.Np * (Y.kfast ? 32 : 8)), 256, 0, s>>>(
        Y, K, g.Kc, g.nch, g.Np, b.ey);
    oz_emax_kernel<<<grid_for(g.Mp), 256, 0, s>>>(b.ex, g.nch, g.Mp, b.exmax);
    oz_emax_kernel<<<grid_for(g.Np), 256, 0, s>>>(b.ey, g.nch, g.Np, b.eymax);
    oz_split_kernel<<<grid_for((long long)g.Mp * g.Kp), 256, 0, s>>>(X, K, g.Kc, g.Kp, g.Mp, b.ex,
                                                                    b.sx);
    oz_split_kernel<<<grid_for((long long)g.Np * g.Kp), 256, 0, s>>>(Y, K, g.Kc, g.Kp, g.Np, b.ey,
                                                                    b.sy);
    static std::atomic<bool> configured[256] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (!configured[dev & 255].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kGemmSmem);
        if (e != cudaSuccess) return e;
        configured[dev & 255].store(true, std::memory_order_release);
    }
    dim3 grid((unsigned)(g.Mp / kBM), (unsigned)(g.Np / kBN), (unsigned)g.splits);
    oz_gemm_kernel<<<grid, kThreads, kGemmSmem, s>>>(b.sx, b.sy, g.Mp, g.Np, g.Kp, g.Kc, g.cps,
                                                     g.nch, b.fold);
    oz_combine_kernel<<<grid_for((long long)g.splits * M * N), 256, 0, s>>>(
        b.fold, b.ex, b.ey, b.exmax, b.eymax, M, N, g.Mp, g.Np, g.cps, g.nch, g.splits, Out,
        out_ld, split_stride);
    count_launch(8);
    return cudaGetLastError();
}

}  // namespace gpp

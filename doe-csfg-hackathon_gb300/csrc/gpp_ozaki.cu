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
//    exponent (max |x| < 2^e), s_1 in [-128, 128] and s_i in [-64, 63]:
//    integers, held exactly in bf16 (8 significant bits).  S = 8 slices keep
//    56 bits of the chunk's largest value;
//  * a product of two slices summed over a chunk of at most 512 k values is
//    an integer below 2^24 in magnitude, which the tensor cores' FP32
//    accumulation adds exactly (checked on the GB300 for sums up to 2^24
//    with operands up to 128, with mma.sync and with tcgen05.mma);
//  * pairs (i, j) with the same i + j = d share the scale 2^(-7 d); those
//    whose worst-case sums still fit in 2^24 are summed in one accumulator
//    (10 groups for the 36 pairs with i + j <= 9), the groups' exact
//    integer sums are stored two to an int32, and a combining pass scales
//    them and adds them in float-float;
//  * pairs with i + j > 9 fall below 2^-56 of the largest products and are
//    left out, as are bits past the 8th slice.
//
// Complex products take the 3M form (Gauss: re = P1 - P2, im = P3 - P1 -
// P2 with P1 = sum xr yr, P2 = sum xi yi, P3 = sum (xr + xi)(yr + yi)), so
// three real splittings and three real products, as in zgemm3m_kernel; the
// result agrees with that FP64 GEMM to about 1e-14 of its values.
//
// The tensor-core kernel is tcgen05-native: tcgen05.mma kind::f16 (bf16 in,
// FP32 accumulate in tensor memory), M = 128 x N = 256 per instruction,
// issued by one thread; operands staged by 1-D bulk copies (the slicing pass
// writes each pipeline stage's operand block contiguously, already in the
// no-swizzle core-matrix layout the MMA descriptors describe) through a
// four-stage mbarrier ring; two TMEM accumulators so four epilogue warps
// drain one group (tcgen05.ld) while the next is being summed.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>

#include "gpp_kernels.h"
#include "gpp_ozaki.h"
#include "gpp_ozaki_split.cuh"

namespace gpp {

namespace {

constexpr int kS = kOzSlices;    // slices per operand value
constexpr int kKcMax = 512;      // k values per chunk (exactness bound)
constexpr int kGroups = 10;      // fold groups per (plane, chunk)
constexpr int kSlots = kGroups / 2;  // stored values per (plane, chunk): groups in pairs

// The tensor-core tile: tcgen05.mma M = 128 (rows of X), N = 256 (rows of
// Y), 64 k per pipeline stage (four K = 16 instructions), four stages.
constexpr int kTM = 128, kTN = 256, kTK = 64, kTStages = 4;
constexpr unsigned kStageA = kTM * kTK * 2, kStageB = kTN * kTK * 2;  // 16 KB, 32 KB
constexpr size_t kTcSmem = (size_t)kTStages * (kStageA + kStageB) + 256;
constexpr int kTcThreads = 192;  // warp 0 loads, warp 1 issues the MMAs, warps 2-5 drain TMEM
constexpr int kTmemCols = 2 * kTN;  // two accumulators of 256 FP32 columns

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
// Groups are stored in pairs (2 s, 2 s + 1) as one exact int32: 128 s_d +
// s_(d+1) for the pairs of consecutive d (2-3, 4-5, 6-7) and s + s' for the
// two halves of d = 8 and of d = 9.  Worst cases over 512 k (group bounds
// 2^23, 2^23; 2^23.3, 2^23.6; 2^23.8, 2^24; and 2^24.2, 2^24.3 for the sums)
// stay below 2^31.  kSlotD: the d whose scale 2^(-7 d) the packed value
// carries.
__constant__ unsigned char kSlotD[kSlots] = {3, 5, 7, 8, 9};
__constant__ unsigned char kSlotShift[kSlots] = {7, 7, 7, 0, 0};  // log2 of the even group's weight

struct Geometry {
    int M, N, K;       // logical sizes
    int Mp, Np;        // padded to the block tile
    int nch, Kc, Kp;   // chunks, chunk length (multiple of kTK), padded K = nch * Kc
    int cps, splits;   // chunks per split, splits
    int slab_tiles;    // row tiles of X per pass (bounds the stored group sums)
};

// The stored group sums of one pass take at most 8 GB (GPP_OZAKI_FOLD_MB
// overrides it, for tests); a larger product runs in passes over slabs of
// X's row tiles.
size_t fold_budget() {
    const char *v = getenv("GPP_OZAKI_FOLD_MB");
    const long long mb = v ? atoll(v) : 0;
    return mb > 0 ? (size_t)mb << 20 : size_t(8) << 30;
}

Geometry geometry(int M, int N, int K, int splits) {
    Geometry g;
    g.M = M;
    g.N = N;
    g.K = K;
    g.Mp = ceil_div(std::max(M, 1), kTM) * kTM;
    g.Np = ceil_div(std::max(N, 1), kTN) * kTN;
    g.nch = std::max(1, ceil_div(K, kKcMax));
    g.Kc = ceil_div(ceil_div(std::max(K, 1), g.nch), kTK) * kTK;
    g.Kp = g.nch * g.Kc;
    g.cps = ceil_div(g.nch, std::max(1, splits));
    g.splits = ceil_div(g.nch, g.cps);
    const size_t per_tile = sizeof(int) * (size_t)g.splits * 3 * g.cps * kSlots * kTM * g.Np;
    g.slab_tiles = (int)std::max<size_t>(1, std::min<size_t>(g.Mp / kTM, fold_budget() / per_tile));
    return g;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

struct Buffers {
    __nv_bfloat16 *sx, *sy;
    int *ex, *ey, *exmax, *eymax;
    int *fold;  // [splits][3][cps][kSlots][slab rows][Np]: group pairs' exact sums, packed
};

size_t fold_elems(const Geometry &g) {
    return (size_t)g.splits * 3 * g.cps * kSlots * ((size_t)g.slab_tiles * kTM) * g.Np;
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
    b.fold = reinterpret_cast<int *>(w);
    return b;
}

__device__ __forceinline__ double2 operand_at(const OzOperand &z, int l, int k) {
    return __ldg(z.kfast ? z.z + (size_t)l * z.ld + k : z.z + (size_t)k * z.ld + l);
}

// Exponent of an all-zero chunk: far enough below any double's that every
// scale formed from it underflows to zero.
constexpr int kZeroExp = -4000;
// Exponent of a chunk holding an Inf or a NaN: its slices are all zero and
// every output of its row or column becomes NaN in the combining pass.
constexpr int kNonFiniteExp = 1 << 20;

// |x| as its bit pattern (monotone in |x| for every double but NaN).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
// A bound on |re|, |im|, |re + im| as bits (no FP64 instruction).
__device__ __forceinline__ unsigned long long max3_bits(double2 v) {
    return max(max(abs_bits(v.x), abs_bits(v.y)), oz_sum_abs_bits(v.x, v.y));
}
// The e of frexp for the nonzero magnitude with bits b (b < 2^e).
__device__ __forceinline__ int exp_of_bits(unsigned long long b) {
    if (b == 0) return kZeroExp;
    const int E = (int)(b >> 52);
    if (E == 0x7FF) return kNonFiniteExp;  // the bit patterns of Inf and NaN are the largest
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

// Slice planes are laid out for the tensor cores: blocks of R rows x kTK k
// (R = kTM for X, kTN for Y), one block per pipeline stage and so one bulk
// copy, ordered (row tile, k step); inside a block the no-swizzle K-major
// core-matrix layout of tcgen05.mma -- core matrices of 8 rows x 16 bytes,
// stored whole (128 bytes), the 8 k-cores of a row group next to each other
// (1024 bytes per row group).  In memory order: row tile, k step, row group
// of 8, k-core, row within the group, k within the core.

// Slices of the three real planes (re, im, re + im): plane (g, i) holds
// s_(i+1) of plane g at (l, k) in that layout; zero outside
// L x K.  The slices are the balanced base-128 digits of
// round(x 2^(7 S - e)): s_2..s_S in [-64, 63], s_1 the rest (|s_1| <= 128),
// so x = 2^e sum_i s_i 2^(-7 i) to within 2^(e - 57).  Integer arithmetic
// throughout (the FP64 pipe is slow on GB300).  A thread per core-matrix row
// (8 consecutive k of one row l), threads in the planes' memory order, so
// each writes one 16-byte chunk per plane and a warp writes 512 contiguous
// bytes.
__global__ void __launch_bounds__(256, 2) oz_split_kernel(OzOperand z, int K, int Kc, int Kp,
                                                          int Lp, int R, const int *E,
                                                          __nv_bfloat16 *out) {
    const long long n = (long long)Lp * (Kp / 8);
    const size_t plane = (size_t)Lp * Kp;
    const int groups = R / 8, ksteps = Kp / kTK;
    for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < n;
         t += (long long)gridDim.x * 256) {
        const int r_lo = (int)(t & 7), j = (int)((t >> 3) & 7);
        const long long q = t >> 6;
        const int rg = (int)(q % groups);
        const long long block = q / groups;
        const int ks = (int)(block % ksteps), rt = (int)(block / ksteps);
        const int l = rt * R + rg * 8 + r_lo, k0 = ks * kTK + j * 8;
        const int e = E[(size_t)(k0 / Kc) * Lp + l];  // one chunk: Kc is a multiple of kTK
        double2 v[8];
#pragma unroll
        for (int kk = 0; kk < 8; ++kk)
            v[kk] = (l < z.L && k0 + kk < K) ? operand_at(z, l, k0 + kk) : make_double2(0.0, 0.0);
#pragma unroll
        for (int g = 0; g < 3; ++g) {
            unsigned packed[kS][4];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                // re and im as fixed-point integers; the re + im plane is their
                // sum (within one unit of round((re + im) 2^(56 - e)), at most
                // 2^56 + 1 in magnitude), formed without an FP64 addition.
                const long long N = g == 0   ? oz_fixed_point(v[kk].x, e)
                                    : g == 1 ? oz_fixed_point(v[kk].y, e)
                                             : oz_fixed_point(v[kk].x, e) + oz_fixed_point(v[kk].y, e);
                int d[kS];
                oz_digits(N, d);
#pragma unroll
                for (int i = 0; i < kS; ++i) {
                    const unsigned short h = __bfloat16_as_ushort(__int2bfloat16_rn(d[i]));
                    if (kk & 1)
                        packed[i][kk >> 1] |= (unsigned)h << 16;
                    else
                        packed[i][kk >> 1] = h;
                }
            }
#pragma unroll
            for (int i = 0; i < kS; ++i)
                *reinterpret_cast<uint4 *>(out + (size_t)(g * kS + i) * plane + (size_t)t * 8) =
                    make_uint4(packed[i][0], packed[i][1], packed[i][2], packed[i][3]);
        }
    }
}

// ---------------------------------------------------------------------------
// tcgen05 / mbarrier primitives.
__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void bar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void bar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool bar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for phase `parity`: gives up after kWaitLimit polls, or as soon
// as another thread of the block raised *abort (and then raises it itself).
__device__ __forceinline__ bool bar_wait(unsigned long long *bar, unsigned parity,
                                         volatile int *abort) {
    for (int it = 0; it < kWaitLimit; ++it) {
        if (bar_try_wait(bar, parity)) return true;
        if ((it & 63) == 63 && *abort) return false;
    }
    *abort = 1;
    return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Shared-memory matrix descriptor of tcgen05.mma for the no-swizzle K-major
// layout: start address, LBO (bytes to the next core matrix along K), SBO
// (bytes to the next 8-row group), the sm_100 descriptor version (bit 46).
__device__ __forceinline__ unsigned long long umma_desc(unsigned saddr, unsigned lbo,
                                                        unsigned sbo) {
    return (unsigned long long)((saddr & 0x3FFFF) >> 4) |
           ((unsigned long long)((lbo >> 4) & 0x3FFF) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1), A and
// B bf16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
constexpr unsigned kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(kTN >> 3) << 17) |
                            ((unsigned)(kTM >> 4) << 24);
__device__ __forceinline__ void umma_bf16(unsigned tmem, unsigned long long a, unsigned long long b,
                                          unsigned accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(unsigned long long *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32]) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// Step t of a block's sequence (plane g, chunk cl of the split, slice pair p,
// k step ks fastest).
struct TcStep {
    int g, cl, p, ks;
};
__device__ __forceinline__ TcStep tc_decode(int t, int KS, int nch_here) {
    TcStep q;
    q.ks = t % KS;
    int r = t / KS;
    q.p = r % kPairs;
    r /= kPairs;
    q.cl = r % nch_here;
    q.g = r / nch_here;
    return q;
}

// The tensor-core products on tcgen05: block (bx, by, z) computes rows
// [128 (mt0 + bx), +128) of X against rows [256 by, +256) of Y over split
// z's chunks, its group sums stored at slab row 128 bx + ... (slab of Ms
// rows), packed in pairs (kSlotD).  Warp 0 (one thread) streams each step's
// two operand blocks into a
// four-stage shared-memory ring with 1-D bulk copies completing on full[s];
// warp 1 (one thread) issues four K = 16 tcgen05.mma per step into one of two
// TMEM accumulators (128 lanes x 256 FP32 columns each) and commits to
// empty[s], and at a group's end to accfull[a]; warps 2-5 read a finished
// accumulator (each warp its 32 TMEM lanes, 32 columns per tcgen05.ld),
// store the group's exact sums as int32 at fold[((((z 3 + g) cps + cl)
// kSlots + group / 2) Ms + m) Np + n] (an odd group packed with the even one
// stored there before it) and release it on accempty[a].  Every wait is
// bounded; a block that gives up records kErrPipelineTimeout, lets its
// copies and MMAs finish and frees its TMEM.
__global__ void __launch_bounds__(kTcThreads, 1)
oz_tc_kernel(const __nv_bfloat16 *__restrict__ SX, const __nv_bfloat16 *__restrict__ SY, int Mp,
             int Np, int Kp, int Kc, int cps, int nch, int mt0, int Ms, int *__restrict__ fold,
             int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;
    unsigned char *sB = smem + (size_t)kTStages * kStageA;
    unsigned long long *bars =
        reinterpret_cast<unsigned long long *>(smem + (size_t)kTStages * (kStageA + kStageB));
    unsigned long long *full = bars, *empty = bars + kTStages;
    unsigned long long *accfull = bars + 2 * kTStages, *accempty = accfull + 2;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(accempty + 2);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    int *issued = abort_flag + 1, *consumed = abort_flag + 2;
    volatile int *abort = abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mt = mt0 + blockIdx.x, nt = blockIdx.y, z = blockIdx.z;
    const int c0 = z * cps, nch_here = min(cps, nch - c0);
    const int KS = Kc / kTK, ksteps = Kp / kTK;
    const int T = 3 * nch_here * kPairs * KS;
    const int NG = 3 * nch_here * kGroups;

    if (tid == 0) {
        for (int s = 0; s < kTStages; ++s) {
            bar_init(&full[s], 1);
            bar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            bar_init(&accfull[a], 1);
            bar_init(&accempty[a], 128);
        }
        *abort_flag = 0;
        *issued = 0;
        *consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // producer
            const size_t xplane = (size_t)Mp * Kp, yplane = (size_t)Np * Kp;
            int t = 0;
            for (; t < T; ++t) {
                const int s = t % kTStages;
                if (t >= kTStages && !bar_wait(&empty[s], ((t / kTStages) - 1) & 1, abort)) break;
                const TcStep q = tc_decode(t, KS, nch_here);
                const int ksg = (c0 + q.cl) * KS + q.ks;
                const __nv_bfloat16 *a = SX + (size_t)(q.g * kS + kPairI[q.p] - 1) * xplane +
                                         ((size_t)mt * ksteps + ksg) * (kTM * kTK);
                const __nv_bfloat16 *b = SY + (size_t)(q.g * kS + kPairJ[q.p] - 1) * yplane +
                                         ((size_t)nt * ksteps + ksg) * (kTN * kTK);
                bar_expect_tx(&full[s], kStageA + kStageB);
                bulk_g2s(sA + (size_t)s * kStageA, a, kStageA, &full[s]);
                bulk_g2s(sB + (size_t)s * kStageB, b, kStageB, &full[s]);
            }
            *issued = t;
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            int G = 0, t = 0;
            for (; t < T; ++t) {
                const int s = t % kTStages;
                const TcStep q = tc_decode(t, KS, nch_here);
                const bool first = q.ks == 0 && (q.p == 0 || kGroupEnd[q.p - 1]);
                const bool last = q.ks == KS - 1 && kGroupEnd[q.p];
                const int a = G & 1;
                if (first && G >= 2 && !bar_wait(&accempty[a], ((G >> 1) - 1) & 1, abort)) break;
                if (!bar_wait(&full[s], (t / kTStages) & 1, abort)) break;
                tc_fence_after();
                const unsigned sa = smem_addr(sA + (size_t)s * kStageA);
                const unsigned sb = smem_addr(sB + (size_t)s * kStageB);
#pragma unroll
                for (int k16 = 0; k16 < kTK / 16; ++k16)
                    umma_bf16(tmem + a * kTN, umma_desc(sa + k16 * 256, 128, 1024),
                              umma_desc(sb + k16 * 256, 128, 1024), !(first && k16 == 0));
                umma_commit(&empty[s]);
                if (last) {
                    umma_commit(&accfull[a]);
                    ++G;
                }
            }
            *consumed = t;
        }
    } else {  // epilogue: warps 2-5, TMEM lanes 32 (warp % 4) ..
        const int quarter = warp & 3;
        const int m = blockIdx.x * kTM + quarter * 32 + lane;  // row within the slab
        const size_t fplane = (size_t)Ms * Np;
        for (int G = 0; G < NG; ++G) {
            const int a = G & 1;
            if (!bar_wait(&accfull[a], (G >> 1) & 1, abort)) break;
            tc_fence_after();
            const int grp = G % kGroups, q = G / kGroups;
            const int cl = q % nch_here, g = q / nch_here;
            const int slot = grp >> 1;
            int *f = fold + ((((size_t)z * 3 + g) * cps + cl) * kSlots + slot) * fplane +
                     (size_t)m * Np + (size_t)nt * kTN;
            const unsigned ta = tmem + ((unsigned)(quarter * 32) << 16) + a * kTN;
            const int shift = kSlotShift[slot];
            if ((grp & 1) == 0) {  // the even group: its sums as they are
#pragma unroll 1
                for (int c = 0; c < kTN; c += 32) {
                    float v[32];
                    tmem_ld32(ta + c, v);
#pragma unroll
                    for (int j = 0; j < 32; j += 4)
                        *reinterpret_cast<int4 *>(f + c + j) =
                            make_int4(__float2int_rn(v[j]), __float2int_rn(v[j + 1]),
                                      __float2int_rn(v[j + 2]), __float2int_rn(v[j + 3]));
                }
            } else {  // the odd group: packed with the even one this thread stored
#pragma unroll 1
                for (int c = 0; c < kTN; c += 32) {
                    int4 e[8];  // read back before the TMEM load, so that the two overlap
#pragma unroll
                    for (int j = 0; j < 8; ++j) e[j] = *reinterpret_cast<const int4 *>(f + c + 4 * j);
                    float v[32];
                    tmem_ld32(ta + c, v);
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        e[j].x = (e[j].x << shift) + __float2int_rn(v[4 * j]);
                        e[j].y = (e[j].y << shift) + __float2int_rn(v[4 * j + 1]);
                        e[j].z = (e[j].z << shift) + __float2int_rn(v[4 * j + 2]);
                        e[j].w = (e[j].w << shift) + __float2int_rn(v[4 * j + 3]);
                        *reinterpret_cast<int4 *>(f + c + 4 * j) = e[j];
                    }
                }
            }
            tc_fence_before();
            bar_arrive(&accempty[a]);
        }
    }

    __syncthreads();
    if (*abort && tid == 0) {
        atomicOr(err, kErrPipelineTimeout);
        // Let the copies still in flight land and the issued MMAs finish.
        for (int t = *consumed; t < *issued; ++t) {
            int spin = 0;
            while (!bar_try_wait(&full[t % kTStages], (unsigned)((t / kTStages) & 1)) &&
                   ++spin < kWaitLimit) {
            }
        }
        if (*consumed > 0) {
            const int t = *consumed - 1;
            int spin = 0;
            while (!bar_try_wait(&empty[t % kTStages], (unsigned)((t / kTStages) & 1)) &&
                   ++spin < kWaitLimit) {
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
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

// (h, l) = (ah + al) + (bh + bl): the heads by TwoSum, exactly; the tails
// and the heads' error added in float (about 2^-47 of the larger operand);
// the pair is left unnormalised for its conversion to a double.
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float &h, float &l) {
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    l = __fadd_rn(__fadd_rn(al, bl), e);
    h = s;
}

// A packed group-pair sum v (|v| < 2^31) as two exact floats hi + lo, hi a
// multiple of 2^16: 2^23 + (v mod 2^16) and 1.5 2^23 + (v >> 16) are built
// from their bits and the offsets taken off (all exact; no conversion
// instruction).
__device__ __forceinline__ void split_packed(int v, float &hi, float &lo) {
    lo = __fsub_rn(__int_as_float(0x4B000000 | (v & 0xFFFF)), 8388608.0f);
    hi = __fmul_rn(__fsub_rn(__int_as_float(0x4B400000 + (v >> 16)), 12582912.0f), 65536.0f);
}


// d 2^e: the exponent field moved when d and the result are normal doubles
// (exact, as scalbn is), a zero returned as it is, scalbn otherwise (off the
// common path).
__device__ __forceinline__ double scale2(double d, int e) {
    const int hi = __double2hiint(d);
    const int ed = (hi >> 20) & 0x7FF;
    if (ed != 0 && ed != 0x7FF && ed + e >= 1 && ed + e <= 2046)
        return __hiloint2double(hi + (e << 20), __double2loint(d));
    if (((hi & 0x7FFFFFFF) | __double2loint(d)) == 0) return d;  // a zero stays itself
    return scalbn(d, e);
}

// The (4 columns, slab row, split) of flat index t.
template <typename I>
__device__ __forceinline__ void combine_cell(I t, I quads, I rows, int &col0, int &r, int &z) {
    col0 = (int)(t % quads) * 4;
    const I q = t / quads;
    r = (int)(q % rows);
    z = (int)(q / rows);
}

// Out = (P1 - P2, P3 - P1 - P2) 2^(Emax_x[m] + Emax_y[n]) per split: each
// plane's packed group sums (split into two exact floats) scaled by
// 2^(e_x - Emax_x + e_y - Emax_y - 7 d) for their chunk and added in
// float-float, in a fixed order; the three planes combined in float-float
// and each result assembled into a double from the bits, with no FP64
// instruction on the common path (the FP64 pipe is the scarce one, and an
// FP64 instruction stalls this pass beside the FP64 occupied-band kernel).
// A thread per (split, row, 4 consecutive columns): the
// stored sums are read as int4 (the padded columns up to Np hold zeros)
// and only columns below N are written.
__global__ void __launch_bounds__(256) oz_combine_kernel(const int *fold, const int *EX,
                                                         const int *EY, const int *EXmax,
                                                         const int *EYmax, int row0, int rows,
                                                         int Ms, int N, int Mp, int Np, int cps,
                                                         int nch, int splits, double2 *Out,
                                                         long long out_ld,
                                                         long long split_stride) {
    const int quads = (N + 3) / 4;
    const long long n = (long long)splits * rows * quads;
    const bool n32 = n < (1ll << 31);  // 32-bit index arithmetic when it fits
    const size_t fplane = (size_t)Ms * Np;
    for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < n;
         t += (long long)gridDim.x * 256) {
        int col0, r, z;  // r: slab row
        if (n32)
            combine_cell<unsigned>((unsigned)t, (unsigned)quads, (unsigned)rows, col0, r, z);
        else
            combine_cell<long long>(t, quads, rows, col0, r, z);
        const int row = row0 + r;
        const int c0 = z * cps, nch_here = min(cps, nch - c0);
        const int exm = __ldg(EXmax + row);
        int eyn[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) eyn[j] = __ldg(EYmax + col0 + j);
        // Each plane's float-float sums: chunk by chunk, slot by slot, the same
        // order for every plane; a chunk's 15 loads are issued together.
        float PH[3][4] = {}, PL[3][4] = {};
        for (int cl = 0; cl < nch_here; ++cl) {
            const int c = c0 + cl;
            const int shx = __ldg(EX + (size_t)c * Mp + row) - exm;
            int sh[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) sh[j] = shx + __ldg(EY + (size_t)c * Np + col0 + j) - eyn[j];
            const int *f = fold + (((size_t)z * 3 * cps + cl) * kSlots) * fplane + (size_t)r * Np + col0;
            int4 v[3][kSlots];
#pragma unroll
            for (int g = 0; g < 3; ++g)
#pragma unroll
                for (int sl = 0; sl < kSlots; ++sl)
                    v[g][sl] = __ldg(reinterpret_cast<const int4 *>(
                        f + ((size_t)g * cps * kSlots + sl) * fplane));
#pragma unroll
            for (int sl = 0; sl < kSlots; ++sl) {
                const int d7 = 7 * kSlotD[sl];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float sc = pow2f(sh[j] - d7);
#pragma unroll
                    for (int g = 0; g < 3; ++g) {
                        const int vv = j == 0 ? v[g][sl].x : j == 1 ? v[g][sl].y : j == 2 ? v[g][sl].z : v[g][sl].w;
                        float hi, lo;
                        split_packed(vv, hi, lo);
                        df_acc(PH[g][j], PL[g][j], __fmul_rn(hi, sc));
                        df_acc(PH[g][j], PL[g][j], __fmul_rn(lo, sc));
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (col0 + j >= N) break;
            const int e = exm + eyn[j];
            // The 3M combination in float-float on the FP32 pipe.
            float rh, rl, bh, bl, ih, il;
            df_add(PH[0][j], PL[0][j], -PH[1][j], -PL[1][j], rh, rl);
            df_add(PH[0][j], PL[0][j], PH[1][j], PL[1][j], bh, bl);
            df_add(PH[2][j], PL[2][j], -bh, -bl, ih, il);
            double2 o = make_double2(scale2(oz_df_to_double(rh, rl), e),
                                     scale2(oz_df_to_double(ih, il), e));
            if (exm >= kNonFiniteExp || eyn[j] >= kNonFiniteExp)
                o = make_double2(__longlong_as_double(0x7FF8000000000000ll),
                                 __longlong_as_double(0x7FF8000000000000ll));
            Out[z * split_stride + (long long)row * out_ld + col0 + j] = o;
        }
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
           align_up(sizeof(int) * fold_elems(g));
}

int ozaki_splits(int K, int splits) { return geometry(1, 1, K, splits).splits; }

cudaError_t ozaki_zgemm(const OzOperand &X, const OzOperand &Y, int M, int N, int K, int splits,
                        double2 *Out, long long out_ld, long long split_stride, void *ws, int *err,
                        cudaStream_t s, cudaEvent_t after_slices) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    const Geometry g = geometry(M, N, K, splits);
    if (g.Mp / kTM > 65535 || g.Np / kTN > 65535 || g.splits > 65535)
        return cudaErrorInvalidConfiguration;
    const Buffers b = carve(g, ws);
    // kfast: a warp per (row, chunk); else a block per (chunk, 32 rows).
    oz_exp_kernel<<<grid_for((long long)g.nch * g.Mp * (X.kfast ? 32 : 8)), 256, 0, s>>>(
        X, K, g.Kc, g.nch, g.Mp, b.ex);
    oz_exp_kernel<<<grid_for((long long)g.nch * g.Np * (Y.kfast ? 32 : 8)), 256, 0, s>>>(
        Y, K, g.Kc, g.nch, g.Np, b.ey);
    oz_emax_kernel<<<grid_for(g.Mp), 256, 0, s>>>(b.ex, g.nch, g.Mp, b.exmax);
    oz_emax_kernel<<<grid_for(g.Np), 256, 0, s>>>(b.ey, g.nch, g.Np, b.eymax);
    oz_split_kernel<<<grid_for((long long)g.Mp * g.Kp / 8), 256, 0, s>>>(X, K, g.Kc, g.Kp, g.Mp,
                                                                        kTM, b.ex, b.sx);
    oz_split_kernel<<<grid_for((long long)g.Np * g.Kp / 8), 256, 0, s>>>(Y, K, g.Kc, g.Kp, g.Np,
                                                                        kTN, b.ey, b.sy);
    cudaError_t e = after_slices ? cudaEventRecord(after_slices, s) : cudaSuccess;
    if (e != cudaSuccess) return e;
    static std::atomic<bool> configured[256] = {};
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (!configured[dev & 255].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(oz_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTcSmem);
        if (e != cudaSuccess) return e;
        configured[dev & 255].store(true, std::memory_order_release);
    }
    // Passes over slabs of X's row tiles, each storing its group sums in the
    // same buffer and combining them into its rows of Out.
    const int mtiles = g.Mp / kTM, Ms = g.slab_tiles * kTM;
    int passes = 0;
    for (int mt0 = 0; mt0 < mtiles; mt0 += g.slab_tiles, ++passes) {
        const int tiles = std::min(g.slab_tiles, mtiles - mt0);
        const int row0 = mt0 * kTM, rows = std::min(M - row0, tiles * kTM);
        dim3 grid((unsigned)tiles, (unsigned)(g.Np / kTN), (unsigned)g.splits);
        oz_tc_kernel<<<grid, kTcThreads, kTcSmem, s>>>(b.sx, b.sy, g.Mp, g.Np, g.Kp, g.Kc, g.cps,
                                                       g.nch, mt0, Ms, b.fold, err);
        if (rows > 0)
            oz_combine_kernel<<<grid_for((long long)g.splits * rows * ceil_div(N, 4)), 256, 0,
                                s>>>(b.fold, b.ex, b.ey, b.exmax, b.eymax, row0, rows, Ms, N,
                                     g.Mp, g.Np, g.cps, g.nch, g.splits, Out, out_ld,
                                     split_stride);
    }
    count_launch(6 + 2 * passes);
    return cudaGetLastError();
}

}  // namespace gpp

// gpp_ozaki_split.cuh -- the integer slicing of gpp_ozaki.cu, host and
// device: an FP64 value x of a chunk with exponent e (every |x| < 2^e) as
// slices s_1..s_S with x = 2^e sum_i s_i 2^(-7 i) to within 2^(e - 57);
// and the other bit-level steps of its passes that keep FP64 instructions
// out of them (a bound on |x + y|, a float-float pair assembled into a
// double).  On GB300 a warp that issues even one FP64 instruction stalls
// while an FP64-bound kernel runs beside it, so these passes use the
// integer pipes only and overlap with such kernels.
#pragma once

#include <cuda_runtime.h>

namespace gpp {

constexpr int kOzSlices = 8;

// round(x 2^(7 S - e)) for |x| < 2^e (ties away from zero), from the
// double's bits with integer operations only: |result| < 2^(7 S) = 2^56, so
// it is exact in 64-bit arithmetic and the left shift never overflows.
__host__ __device__ __forceinline__ long long oz_fixed_point(double x, int e) {
    unsigned long long u;
#ifdef __CUDA_ARCH__
    u = (unsigned long long)__double_as_longlong(x);
#else
    __builtin_memcpy(&u, &x, sizeof u);
#endif
    const int E = (int)((u >> 52) & 0x7FF);
    unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    if (E == 0 && m == 0) return 0;
    int ex = -1074;  // x = m 2^ex
    if (E > 0) {
        m |= 1ull << 52;
        ex = E - 1075;
    }
    const int sh = ex + 7 * kOzSlices - e;
    unsigned long long N;
    if (sh >= 0)
        N = m << sh;
    else if (sh > -64)
        N = (m + (1ull << (-sh - 1))) >> (-sh);
    else
        N = 0;
    return (u >> 63) ? -(long long)N : (long long)N;
}

// The balanced base-128 digits of oz_fixed_point(x, e), most significant
// first: d[1..S-1] in [-64, 63], d[0] the rest (|d[0]| <= 128).  Integers of
// at most 8 significant bits, so exact in bf16.
// The balanced base-128 digits of a fixed-point value N, |N| <= 2^56 + 1:
// d_2..d_8 in [-64, 63] and d_1 the rest, N = sum_i d_i 128^(8 - i).  With
// B = 64 (1 + 128 + ... + 128^6), M = N + B has the plain base-128 digits
// d_i + 64 below its top (floor) digit d_1, so every digit is a shift and a
// mask of M, without the carry chain of peeling them off one by one (the
// representation is unique, so the digits are the same).
constexpr long long kOzBalance = 64 * (((1ll << 49) - 1) / 127);
__host__ __device__ __forceinline__ void oz_digits(long long N, int (&d)[kOzSlices]) {
    const long long M = N + kOzBalance;
#pragma unroll
    for (int i = 1; i < kOzSlices; ++i) d[i] = (int)((M >> (7 * (kOzSlices - 1 - i))) & 127) - 64;
    d[0] = (int)(M >> (7 * (kOzSlices - 1)));
}

__host__ __device__ __forceinline__ void oz_slices(double x, int e, int (&d)[kOzSlices]) {
    oz_digits(oz_fixed_point(x, e), d);
}

__host__ __device__ __forceinline__ unsigned long long oz_bits(double x) {
    unsigned long long u;
#ifdef __CUDA_ARCH__
    u = (unsigned long long)__double_as_longlong(x);
#else
    __builtin_memcpy(&u, &x, sizeof u);
#endif
    return u;
}
__host__ __device__ __forceinline__ double oz_double(unsigned long long u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    __builtin_memcpy(&x, &u, sizeof x);
    return x;
#endif
}
__host__ __device__ __forceinline__ unsigned oz_fbits(float x) {
    unsigned u;
#ifdef __CUDA_ARCH__
    u = __float_as_uint(x);
#else
    __builtin_memcpy(&u, &x, sizeof u);
#endif
    return u;
}

// The bit pattern of a double >= |x + y|: for x and y of one sign, |x| + |y|
// rounded up from their aligned mantissas; for opposite signs 0, since then
// |x + y| <= max(|x|, |y|).  A non-finite operand gives its own bits (at
// least those of Inf), a sum past the largest double those of Inf, as the
// FP64 sum would.
__host__ __device__ __forceinline__ unsigned long long oz_sum_abs_bits(double x, double y) {
    const unsigned long long kAbs = 0x7FFFFFFFFFFFFFFFull, kMant = 0xFFFFFFFFFFFFFull;
    const unsigned long long ux = oz_bits(x), uy = oz_bits(y);
    if ((ux ^ uy) >> 63) return 0;
    unsigned long long a = ux & kAbs, b = uy & kAbs;
    if (a < b) {
        const unsigned long long t = a;
        a = b;
        b = t;
    }
    if ((a >> 52) == 0x7FF || b == 0) return a;
    const int Ea = (int)(a >> 52), Eb = (int)(b >> 52);
    const unsigned long long ma = (a & kMant) | (Ea ? 1ull << 52 : 0);
    const unsigned long long mb = (b & kMant) | (Eb ? 1ull << 52 : 0);
    const int ea = Ea > 1 ? Ea : 1, d = ea - (Eb > 1 ? Eb : 1);  // a >= b, so d >= 0
    const unsigned long long mbs =
        d >= 64 ? 1ull : (mb >> d) + ((mb & ((1ull << d) - 1)) != 0);  // rounded up
    unsigned long long S = ma + mbs;  // (|x| + |y|) 2^(1074 - ea + 1), rounded up; < 2^54
    int E = ea;
    if (S >> 53) {
        S = (S >> 1) + (S & 1);
        ++E;
        if (S >> 53) {
            S >>= 1;
            ++E;
        }
    }
    if (E >= 0x7FF) return 0x7FF0000000000000ull;
    if (!(S >> 52)) return S;  // below the normal range: E == 1, the subnormal pattern
    return ((unsigned long long)E << 52) | (S & kMant);
}

// The double h + l of a normalised float-float pair (|l| <= ulp(h) / 2),
// assembled from the bits: h's mantissa moved up 29 bits plus l in units of
// 2^-29 of h's last place (rounded; when h is a power of two and l is of the
// other sign, one bit of l is lost); within one unit in the last place.
// Zero gives a signed zero; *ok is cleared for a subnormal or non-finite h,
// which the caller converts in FP64 instead.
__host__ __device__ __forceinline__ double oz_pair_to_double(float h, float l, bool *ok) {
    const unsigned uh = oz_fbits(h), ul = oz_fbits(l);
    const int eh = (int)((uh >> 23) & 0xFFu), el = (int)((ul >> 23) & 0xFFu);
    *ok = true;
    if ((uh & 0x7FFFFFFFu) == 0) return oz_double((unsigned long long)(uh >> 31) << 63);
    if (eh == 0 || eh == 0xFF) {
        *ok = false;
        return 0.0;
    }
    long long D = (long long)((uh & 0x7FFFFFu) | 0x800000u) << 29;  // h in units of 2^(eh - 179)
    if ((ul & 0x7FFFFFFFu) != 0 && el != 0xFF) {
        // l = ml 2^(el' - 150), el' = 1 and no leading bit for a subnormal l
        const long long ml = (long long)((ul & 0x7FFFFFu) | (el ? 0x800000u : 0u));
        const int sh = (el ? el : 1) - eh + 29;  // <= 5 for a normalised pair
        long long L = 0;
        if (sh >= 0)
            L = ml << sh;
        else if (sh > -40)
            L = (ml + (1ll << (-sh - 1))) >> (-sh);
        D += ((uh ^ ul) >> 31) ? -L : L;
    }
    int e = eh + 896;  // the double's exponent field while D is in [2^52, 2^53)
    if (D >= (1ll << 53)) {
        D = (D + 1) >> 1;
        ++e;
    } else if (D < (1ll << 52)) {
        D <<= 1;
        --e;
    }
    if (D >= (1ll << 53)) {
        D >>= 1;
        ++e;
    }
    return oz_double(((unsigned long long)(uh >> 31) << 63) | ((unsigned long long)e << 52) |
                     ((unsigned long long)D & 0xFFFFFFFFFFFFFull));
}

// The double of any float-float pair h + l: renormalised by TwoSum (exact),
// then assembled from the bits; FP64 only for a subnormal or non-finite head.
__host__ __device__ __forceinline__ double oz_df_to_double(float h, float l) {
#ifdef __CUDA_ARCH__
    const float s = __fadd_rn(h, l);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(l, bb));
#else
    const float s = h + l;
    const float bb = s - h;
    const float e = (h - (s - bb)) + (l - bb);
#endif
    bool ok;
    const double d = oz_pair_to_double(s, e, &ok);
    return ok ? d : (double)s + (double)e;
}

}  // namespace gpp

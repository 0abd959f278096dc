// gpp_df.cuh -- float-float ("df") arithmetic for the mixed-precision GPP
// kernels.  A df value is the unevaluated sum h + l of two floats (~48
// significant bits).  Building blocks are the error-free transformations
// TwoSum (Knuth, TAOCP vol. 2, 4.2.2) and FMA-based TwoProduct (Ogita, Rump &
// Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).
// Results are left unnormalised (|l| may exceed half an ulp of h): every
// later operation consumes h and l separately, so the only rounding that is
// not captured exactly is second order (~2^-47 of the operands).
#pragma once

#include <cuda_runtime.h>

#include <cstring>

namespace gpp {

struct df {
    float h, l;
};

// Additions and products that the compiler must not fuse into FMAs: nvcc
// contracts a*b + c by default, which would silently break the error-free
// transformations below (TwoSum relies on s = fl(a + b) of the already
// rounded operands).  The _rn intrinsics are never contracted.
__host__ __device__ __forceinline__ float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ __forceinline__ float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

__host__ __device__ __forceinline__ df two_sum(float a, float b) {
    const float s = fadd(a, b);
    const float bb = fsub(s, a);
    const float e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
    return {s, e};
}
// (a.h + a.l) * (b.h + b.l) without the l*l term.
__host__ __device__ __forceinline__ df df_mul(df a, df b) {
    const float p = fmul(a.h, b.h);
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return {p, e};
}
__host__ __device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.h, b.h);
    s.l = fadd(s.l, fadd(a.l, b.l));
    return s;
}
__host__ __device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, {-b.h, -b.l}); }
__host__ __device__ __forceinline__ df df_sqr(df a) {
    const float p = fmul(a.h, a.h);
    float e = fmaf(a.h, a.h, -p);
    e = fmaf(fadd(a.h, a.h), a.l, e);
    return {p, e};
}
// Renormalise so that |l| <= ulp(h)/2 (Fast2Sum, Dekker 1971).  Needed after
// a cancelling subtraction, where l can be a sizeable fraction of h and the
// l*l terms that df_mul / df_sqr drop would no longer be negligible.  The
// exponent precondition of Fast2Sum can only fail when |h| is within a few
// ulps of zero, where the absolute error it leaves is itself a few ulps of l.
__host__ __device__ __forceinline__ df df_norm(df a) {
    const float s = fadd(a.h, a.l);
    return {s, fsub(a.l, fsub(s, a.h))};
}
// 1/d for a normalised d: hardware reciprocal seed r of d.h (MUFU, relative
// error ~2^-23) and a second-order Newton-Raphson correction r (e + e^2),
// e = 1 - d r computed against the full df value; error ~2^-45 and, unlike
// the first-order step (always short by r e^2), without a sign preference
// that long sums would accumulate.
__host__ __device__ __forceinline__ df df_rcp(df d) {
    float r;
#ifdef __CUDA_ARCH__
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d.h));
#else
    r = 1.0f / d.h;
#endif
    float e = fmaf(-d.h, r, 1.0f);
    e = fmaf(-d.l, r, e);
    e = fmaf(e, e, e);
    return {r, fmul(r, e)};
}
__host__ __device__ __forceinline__ df split(double x) {
#ifdef __CUDA_ARCH__
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
#else
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
#endif
}
__host__ __device__ __forceinline__ double to_double(df a) { return (double)a.h + (double)a.l; }


// Small integer k (|k| < 2^22) to float, exactly, without a conversion
// instruction: 1.5 * 2^23 + k has k in its low mantissa bits.
__host__ __device__ __forceinline__ float small_int_to_float(int k) {
    const unsigned u = 0x4B400000u + (unsigned)k;
    float f;
    memcpy(&f, &u, 4);
    return fsub(f, 12582912.0f);
}
// split(x) from the bits of x with integer and FP32 operations, for the prep
// kernels that split gigabytes of inputs: on GB300 the FP64 conversions and
// subtraction of split(), and integer-to-float conversions too, run on the
// narrow FP64 pipe.  With x = (2^52 + m) 2^(e-1075): h keeps the top 23 bits
// of m, rounded to nearest even on the low 29; x - h = r 2^(e-1075) exactly,
// with r the signed remainder (|r| <= 2^28).  Writing r = rh 2^14 + rl, both
// parts exact floats, l = fma(rh, 2^(e-1061), rl 2^(e-1075)) rounds r
// 2^(e-1075) once, as split() does.  Same bits as split() wherever h and l
// are normal floats; exponents outside [2^-60, 2^48] (zero, subnormal, huge,
// Inf, NaN) take split().
// The out-of-range case, kept out of line so that the compiler cannot
// hoist its FP64 conversions into the common path.
#ifdef __CUDA_ARCH__
__device__ __noinline__ df split_far(double x) { return split(x); }
#else
inline df split_far(double x) { return split(x); }
#endif
__host__ __device__ __forceinline__ df split_bits(double x) {
    unsigned long long b;
#ifdef __CUDA_ARCH__
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));  // opaque: no FP compare for the range test
#else
    memcpy(&b, &x, 8);
#endif
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 60 || e > 1023 + 48) return split_far(x);
    const unsigned mhi = (unsigned)(b >> 29) & 0x7fffffu;  // mantissa bits 51..29
    const unsigned rem = (unsigned)b & 0x1fffffffu;         // mantissa bits 28..0
    const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (mhi & 1u))) ? 1u : 0u;
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    // A carry out of the mantissa moves h to the next binade, as rounding does.
    const unsigned hb = sign | ((((unsigned)(e - 1023 + 127) << 23) | mhi) + up);
    const int r = (int)rem - (int)(up << 29);
    const float rh = small_int_to_float(r >> 14), rl = small_int_to_float(r & 0x3fff);
    const unsigned sb = (unsigned)(e - 1075 + 127) << 23;  // 2^(e-1075), a normal float
    const unsigned sb14 = sb + (14u << 23);                // 2^(e-1061)
    float h, scale, scale14;
    memcpy(&h, &hb, 4);
    memcpy(&scale, &sb, 4);
    memcpy(&scale14, &sb14, 4);
    const float l = fmaf(rh, scale14, fmul(rl, scale));
    return {h, (sign && r != 0) ? -l : l};  // +0 for an exact x, as split() gives
}

}  // namespace gpp

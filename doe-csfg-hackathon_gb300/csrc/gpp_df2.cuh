// gpp_df2.cuh -- two float-float ("df") lanes per operation, on the packed
// FP32 instructions of sm_100+ (add/sub/mul/fma .f32x2: one instruction
// issues two independent FP32 operations).  A df2 value holds two df numbers
// in structure-of-arrays form, {h.x + l.x, h.y + l.y}, so every step of the
// df algorithms in gpp_df.cuh becomes one packed instruction for both lanes.
// Per lane the results are bit-identical to the scalar df functions: the
// packed operations round each component exactly like __fadd_rn, __fmul_rn
// and __fmaf_rn, and like those they are never contracted by the compiler.
#pragma once

#include <cuda_runtime.h>

#include "gpp_df.cuh"

namespace gpp {

struct df2 {
    float2 h, l;
};

__host__ __device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__host__ __device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }

__host__ __device__ __forceinline__ float2 f2add(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
// a - b as a + (-b): exact negation folds into the packed add's operand, and
// (unlike an inline-asm sub.f32x2) lets a lane-broadcast operand be read
// without first copying it into a register pair.
__host__ __device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
__host__ __device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __fmul2_rn(a, b);
#else
    return make_float2(a.x * b.x, a.y * b.y);
#endif
}
__host__ __device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
#ifdef __CUDA_ARCH__
    return __ffma2_rn(a, b, c);
#else
    return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}

// Both lanes hold the same df value.
__host__ __device__ __forceinline__ df2 df2_bcast(df a) { return {f2(a.h, a.h), f2(a.l, a.l)}; }
__host__ __device__ __forceinline__ df df2_lane(const df2 &a, int i) {
    return i == 0 ? df{a.h.x, a.l.x} : df{a.h.y, a.l.y};
}
__host__ __device__ __forceinline__ void df2_set_lane(df2 &a, int i, df v) {
    if (i == 0) {
        a.h.x = v.h;
        a.l.x = v.l;
    } else {
        a.h.y = v.h;
        a.l.y = v.l;
    }
}

// TwoSum (Knuth) on both lanes.
__host__ __device__ __forceinline__ df2 two_sum2(float2 a, float2 b) {
    const float2 s = f2add(a, b);
    const float2 bb = f2sub(s, a);
    const float2 e = f2add(f2sub(a, f2sub(s, bb)), f2sub(b, bb));
    return {s, e};
}
__host__ __device__ __forceinline__ df2 df2_add(const df2 &a, const df2 &b) {
    df2 s = two_sum2(a.h, b.h);
    s.l = f2add(s.l, f2add(a.l, b.l));
    return s;
}
// TwoSum of a + (-b), written without the negation; per lane bit-identical
// to two_sum(a, -b).
__host__ __device__ __forceinline__ df2 two_diff2(float2 a, float2 b) {
    const float2 s = f2sub(a, b);
    const float2 bb = f2sub(s, a);
    const float2 e = f2sub(f2sub(a, f2sub(s, bb)), f2add(b, bb));
    return {s, e};
}
__host__ __device__ __forceinline__ df2 df2_sub(const df2 &a, const df2 &b) {
    df2 s = two_diff2(a.h, b.h);
    s.l = f2add(s.l, f2sub(a.l, b.l));
    return s;
}
// (a.h + a.l)(b.h + b.l) without the l*l term (FMA TwoProduct for h*h).
__host__ __device__ __forceinline__ df2 df2_mul(const df2 &a, const df2 &b) {
    const float2 p = f2mul(a.h, b.h);
    float2 e = f2fma(a.h, b.h, f2neg(p));
    e = f2fma(a.h, b.l, e);
    e = f2fma(a.l, b.h, e);
    return {p, e};
}
// (h + l)^2 for a normalised value (the l*l term, below 2^-48 of the
// result, is left out).
__host__ __device__ __forceinline__ df2 df2_sqr(const df2 &a) {
    const float2 p = f2mul(a.h, a.h);
    float2 e = f2fma(a.h, a.h, f2neg(p));
    e = f2fma(f2add(a.h, a.h), a.l, e);
    return {p, e};
}
// Renormalise both lanes so that |l| <= ulp(h)/2 (Fast2Sum, Dekker 1971),
// after a cancelling subtraction.  Products of an unnormalised operand drop
// an l*l term that is then no longer negligible, and on sums of ~1e10 terms
// that small, one-signed error shows up at the 1e-10 level.
__host__ __device__ __forceinline__ df2 df2_norm(const df2 &a) {
    const float2 s = f2add(a.h, a.l);
    return {s, f2sub(a.l, f2sub(s, a.h))};
}
// 1/d per lane: hardware reciprocal seed r of d.h (MUFU, relative error
// below ~2^-23) and a second-order Newton-Raphson correction,
// r (1 + e + e^2) with e = 1 - d r computed against the full df value.  The
// first-order step alone leaves a one-signed error of -e^2, which long sums
// would accumulate.
__host__ __device__ __forceinline__ df2 df2_rcp(const df2 &d) {
    float2 r;
#ifdef __CUDA_ARCH__
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.x) : "f"(d.h.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.y) : "f"(d.h.y));
#else
    r = make_float2(1.0f / d.h.x, 1.0f / d.h.y);
#endif
    float2 e = f2fma(f2neg(d.h), r, f2(1.0f, 1.0f));
    e = f2fma(f2neg(d.l), r, e);
    e = f2fma(e, e, e);
    return {r, f2mul(r, e)};
}

// The reciprocal 1/d of df2_rcp in two parts, the seed r0 and the
// correction factor c = e + e^2 (1/d = r0 (1 + c) to ~2^-45), for
// df2_mul_rcp: a product by 1/d then needs no separate low part r0 c.
__host__ __device__ __forceinline__ void df2_rcp_parts(const df2 &d, float2 &r0, float2 &c) {
#ifdef __CUDA_ARCH__
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0.x) : "f"(d.h.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0.y) : "f"(d.h.y));
#else
    r0 = make_float2(1.0f / d.h.x, 1.0f / d.h.y);
#endif
    float2 e = f2fma(f2neg(d.h), r0, f2(1.0f, 1.0f));
    e = f2fma(f2neg(d.l), r0, e);
    c = f2fma(e, e, e);
}
// a / d = a r0 (1 + c) in df: p = a.h r0 with its exact rounding error, plus
// the correction p c and the low part a.l r0.  p c stands for a.h r0 c
// (their difference, 2^-24 of a term already 2^-22 small, is far below the
// df rounding); four packed instructions, as df2_mul(a, {r0, r0 c}) costs
// after the extra one that forms r0 c.
__host__ __device__ __forceinline__ df2 df2_mul_rcp(const df2 &a, float2 r0, float2 c) {
    const float2 p = f2mul(a.h, r0);
    float2 e = f2fma(a.h, r0, f2neg(p));
    e = f2fma(p, c, e);
    e = f2fma(a.l, r0, e);
    return {p, e};
}

}  // namespace gpp

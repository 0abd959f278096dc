// gpp_ozaki_split.cuh -- the integer slicing of gpp_ozaki.cu, host and
// device: an FP64 value x of a chunk with exponent e (every |x| < 2^e) as
// slices s_1..s_S with x = 2^e sum_i s_i 2^(-7 i) to within 2^(e - 57).
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
__host__ __device__ __forceinline__ void oz_slices(double x, int e, int (&d)[kOzSlices]) {
    long long N = oz_fixed_point(x, e);
#pragma unroll
    for (int i = kOzSlices - 1; i >= 1; --i) {
        d[i] = (int)((N + 64) & 127) - 64;
        N = (N - d[i]) >> 7;
    }
    d[0] = (int)N;
}

}  // namespace gpp

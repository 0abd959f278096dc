// gpp_ozaki.h -- FP64-class complex GEMM on the tensor cores (gpp_ozaki.cu).
#pragma once

#include <cuda_runtime.h>

#include "gpp_gb300.h"

namespace gpp {

// One complex FP64 operand Z(l, k), l < L, k < K: Z[l * ld + k] when kfast,
// else Z[k * ld + l].
struct OzOperand {
    const double2 *z;
    long long ld;
    bool kfast;
    int L;
};

// Workspace bytes of ozaki_zgemm for an M x N output over K with `splits`
// k splits (split partial results are written separately).
size_t ozaki_bytes(int M, int N, int K, int splits);

// Number of k splits ozaki_zgemm makes of K when asked for `splits` (at most
// `splits`; the k range is cut at chunk boundaries).
int ozaki_splits(int K, int splits);

// Out[z * split_stride + m * out_ld + n] = sum over split z's k range of
// X(m, k) Y(n, k), complex, for m < M, n < N: the k range cut into `splits`
// contiguous parts (as zgemm3m_kernel cuts it, so split partials can be
// added in split order by the caller).  Accuracy is that of an FP64 3M-form
// GEMM; the products run on the tensor cores (tcgen05).  A block whose
// bounded pipeline wait ran out sets kErrPipelineTimeout in *err.
// after_slices, when given, is recorded on s once the slicing passes are
// queued (before the tensor-core passes).
cudaError_t ozaki_zgemm(const OzOperand &X, const OzOperand &Y, int M, int N, int K, int splits,
                        double2 *Out, long long out_ld, long long split_stride, void *ws, int *err,
                        cudaStream_t s, cudaEvent_t after_slices = nullptr);

}  // namespace gpp

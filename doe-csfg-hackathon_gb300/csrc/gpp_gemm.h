// gpp_gemm.h -- the band-independent-frequency FP64 path of the unoccupied
// bands (gpp_gemm.cu): the band sum as one complex GEMM.
#pragma once

#include <cuda_runtime.h>

#include "gpp_gb300.h"
#include "gpp_kernels.h"

namespace gpp {

// Whether this host thread's FP64 GEMMs run on the tensor cores (the Ozaki
// split of gpp_ozaki.cu, the default) rather than on the FP64 pipe
// (zgemm3m_kernel, gpp_set_gemm_path(2)).
bool fp64_gemm_on_tensor_cores();

// Workspace bytes of the GEMM path for `bands` unoccupied bands.
size_t gemm_bytes(const Problem &p, int bands, bool want_n1);

// Unoccupied bands [b0, b1) of a problem with wx_stride == 0, in three
// steps on stream s, each over every G' row so that the results do not
// depend on how a caller splits the rows:
//  1. gemm_band_sum: c and G = sum_n1 c aqsn (needs the band arrays only);
//  2. gemm_rows: for row tiles `rows`, the achtemp partial of each row tile
//     (slot part.ach_tile0 + row tile) -- needs those rows' wtilde/I_eps;
//  3. gemm_per_band: when part.n1 is set (nw >= 3), the per-band partials
//     of acht_n1_loc -- needs every row.
// `ws` holds gemm_bytes(p, b1 - b0, part.n1 != nullptr).
// after_slices: recorded on s once the tensor-core GEMM's slicing passes are
// queued (at the end of the call on the FP64-pipe path).
gpp_status gemm_band_sum(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                         cudaStream_t s, cudaEvent_t after_slices = nullptr);
gpp_status gemm_rows(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                     cudaStream_t s, RowTiles rows = RowTiles());
// split_ws: the mixed path's split planes; M_2 is then formed in float-float
// from them (mixed_m2_fp64) instead of in FP64.
gpp_status gemm_per_band(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                         cudaStream_t s, void *split_ws = nullptr);

// G (ng x nc, FP64) inside a workspace of gemm_bytes(p, bands, want_n1),
// written by gemm_band_sum.
const double2 *gemm_g(const Problem &p, void *ws, int bands, bool want_n1);

}  // namespace gpp

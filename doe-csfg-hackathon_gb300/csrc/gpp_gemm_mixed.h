// gpp_gemm_mixed.h -- the band-independent-frequency mixed-precision path of
// the unoccupied bands (gpp_gemm_mixed.cu): the band sum as a float-float
// complex GEMM.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>

#include "gpp_gb300.h"
#include "gpp_kernels.h"

namespace gpp {

// Workspace bytes for `bands` unoccupied bands.
size_t mixed_gemm_bytes(const Problem &p, int bands, bool want_n1);

// Unoccupied bands [b0, b1) of a problem with wx_stride == 0 on the
// float-float split planes at `split_ws` (bands and wx split for [b0, b1),
// rows split before mixed_gemm_rows reads them):
//  1. mixed_gemm_band_sum: c and G = sum_n1 c aqsn over every G' row;
//  2. mixed_gemm_rows: for row tiles `rows`, each row tile's achtemp partial
//     (slot part.ach_tile0 + row tile);
//  3. mixed_gemm_per_band: when part.n1 is set (nw >= 3), the per-band
//     partials of acht_n1_loc -- H = aqsn M_2^T in float-float over every
//     row (needs every row split).
gpp_status mixed_gemm_band_sum(const Problem &p, const Partials &part, void *split_ws, void *ws,
                               int b0, int b1, cudaStream_t st);
gpp_status mixed_gemm_rows(const Problem &p, const Partials &part, void *split_ws, void *ws, int b0,
                           int b1, cudaStream_t st, RowTiles rows = RowTiles());
gpp_status mixed_gemm_per_band(const Problem &p, const Partials &part, void *split_ws, void *ws,
                               int b0, int b1, cudaStream_t st);

// Step 1 from an FP64 G (ng x nc) computed elsewhere (the tensor-core band
// sum of gpp_gemm.cu): G split into the float-float row-pair planes that
// mixed_gemm_rows reads, in `ws` of mixed_gemm_bytes(p, b1 - b0, false).
gpp_status mixed_gemm_planes_from(const Problem &p, void *ws, int b0, int b1, const double2 *G,
                                  cudaStream_t st);

// M_2 = Q conj(wdiff) / |wdiff|^2 at iw = 2 (the per-band product's right
// operand) as FP64 rows M[r][ig], computed in float-float from the split row
// planes (FP64 within 1e-3 |wx| of the pole) with wx of band wx_band: the
// mixed path's operand of the tensor-core per-band GEMM.
gpp_status mixed_m2_fp64(const Problem &p, void *split_ws, int wx_band, double2 *M,
                         cudaStream_t st);

}  // namespace gpp

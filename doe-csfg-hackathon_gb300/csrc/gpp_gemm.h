// gpp_gemm.h -- the band-independent-frequency FP64 path of the unoccupied
// bands (gpp_gemm.cu): the band sum as one complex GEMM.
#pragma once

#include <cuda_runtime.h>

#include "gpp_gb300.h"
#include "gpp_kernels.h"

namespace gpp {

// Workspace bytes of launch_noflag_gemm for `bands` unoccupied bands.
size_t gemm_bytes(const Problem &p, int bands, bool want_n1);

// Unoccupied bands [b0, b1) of a problem with wx_stride == 0: one achtemp
// partial per row tile (slot part.ach_tile0 + row tile) and, when part.n1 is
// set, per-band partials (nw >= 3).  `ws` holds gemm_bytes(p, b1 - b0, ...).
gpp_status launch_noflag_gemm(const Problem &p, const Partials &part, void *ws, int b0, int b1,
                              cudaStream_t s, RowTiles rows = RowTiles());

}  // namespace gpp

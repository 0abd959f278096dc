// gpp_kernels.h -- host-side launchers of the GPP sigma kernels (internal to
// libgpp_gb300.so; the public C ABI is include/gpp_gb300.h).
#pragma once

#include <cuda_runtime.h>

#include "gpp_gb300.h"
#include "gpp_internal.cuh"

namespace gpp {

// Tile geometry of one family of sigma kernels.  Blocks cover RG local G'
// rows x RN bands x NWC frequencies; the block's threads stride over ig.
struct TileShape {
    int rn, rg, nwc, threads;
};

// Shapes the launchers will use for this problem (also needed to size the
// partial-sum workspace before launching).
TileShape fp64_noflag_shape(const Problem &p);
TileShape flag_shape(const Problem &p);

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// A range of row tiles [begin, end).  Every kernel family tiles G' rows in
// pairs (RG = 2), so a row-pair range means the same rows to all of them;
// the default covers every row.  Launches over parts of the rows write the
// same partial slots as one launch over all of them.
struct RowTiles {
    int begin = 0, end = -1;  // end < 0: to the last row tile
    RowTiles clip(int row_tiles) const {
        RowTiles r;
        r.begin = begin < 0 ? 0 : (begin > row_tiles ? row_tiles : begin);
        r.end = (end < 0 || end > row_tiles) ? row_tiles : end;
        return r;
    }
};

// Unoccupied bands [band_begin, band_end), FP64.  Writes one ach partial per
// (row tile, band tile) block and, when part.n1 is set, per-band partials.
cudaError_t launch_noflag_fp64(const Problem &p, const Partials &part, int band_begin,
                               int band_end, cudaStream_t s, RowTiles rows = RowTiles());
// Occupied bands [0, nvband): full ssxt_scht_solver branch logic in FP64.
// blocks_per_sm > 0 with a device counter `next` (band-independent
// frequencies only): a persistent grid of that many blocks per SM taking row
// tiles from the counter (zeroed on `s` first), for a launch beside the
// tensor-core GEMM (GPP_FLAG_BLOCKS_PER_SM overrides blocks_per_sm).
cudaError_t launch_flag_fp64(const Problem &p, const Partials &part, cudaStream_t s,
                             RowTiles rows = RowTiles(), int blocks_per_sm = 0,
                             int *next = nullptr);
// Static term (reduce_achstemp) over all bands: one partial per block.
int achstemp_blocks(const Problem &p);
cudaError_t launch_achstemp(const Problem &p, double2 *partials, int *err, cudaStream_t s);

// Fixed-order sum of segments: dst[s] (=|+=) sum_{t<len} src[s*stride + t].
struct ReduceOut {
    double2 *c;      // complex destination (or null)
    double *re;      // split destination, always accumulated (or null)
    double *im;
    int accumulate;  // for c: 1 adds into c[s], 0 overwrites
};
cudaError_t launch_reduce(const double2 *src, long long stride, int len, int nseg, ReduceOut out,
                          cudaStream_t s);

// Host-to-device transfer by the SMs (host_pull_kernel): src_dev is the
// device's address of device-accessible host memory; 16-byte aligned
// pointers and a size that is a multiple of 16.
cudaError_t launch_host_pull(void *dst, const void *src_dev, size_t bytes, cudaStream_t s);

// FMA throughput probe (see gpp_probe_fma_peaks).
cudaError_t probe_fma_peaks(double *fp64_tflops, double *fp32_tflops);

// Mixed precision path (gpp_mixed.cu).
size_t mixed_split_bytes(const Problem &p);
// Tile shape of a variant of the unoccupied-band kernel (the default
// variant's for one not compiled for this problem's frequency chunk), and
// whether the variant is compiled for `nw` frequencies.
TileShape mixed_noflag_shape(const Problem &p, int variant);
bool mixed_variant_valid(int variant, int nw);
// The split planes must have been written (launch_split) for the bands used:
// [band_begin, band_end) for the unoccupied kernel, [0, nvband) for the
// occupied one.
cudaError_t launch_mixed_noflag(const Problem &p, const Partials &part, void *split_ws,
                                int band_begin, int band_end, cudaStream_t s, int variant,
                                RowTiles rows = RowTiles());
// blocks_per_sm and next as for launch_flag_fp64.
cudaError_t launch_flag_mixed(const Problem &p, const Partials &part, void *split_ws,
                              cudaStream_t s, RowTiles rows = RowTiles(), int blocks_per_sm = 0,
                              int *next = nullptr);
// Blocks per SM of a persistent occupied-band grid (0: one block per tile);
// GPP_FLAG_BLOCKS_PER_SM, read on every call, overrides the caller's choice.
int flag_blocks_per_sm(int asked);
// One block that waits on an mbarrier nothing arrives at and records the
// bounded-wait timeout in *err (exercises the failure path without a fault).
cudaError_t launch_wait_selftest(int *err, int polls, cudaStream_t s);
// Pipeline variants of the mixed kernel, selectable per call (autotuner).
int mixed_variant_count();
const char *mixed_variant_name(int variant);
int mixed_default_variant();

// Float-float split planes of one state (prep pass of the mixed path).
struct SplitPlanes;
SplitPlanes split_planes_at(const Problem &p, void *split_ws);
cudaError_t launch_split(const Problem &p, void *split_ws, int band_begin, int band_end,
                         cudaStream_t s);
// The same in two steps: the bands (and the reset of the row masks), then
// the rows of a range of row pairs; every row pair must be split before the
// tiles that read it.
cudaError_t launch_split_bands(const Problem &p, void *split_ws, int band_begin, int band_end,
                               cudaStream_t s);
cudaError_t launch_split_rows(const Problem &p, void *split_ws, RowTiles pairs, cudaStream_t s);

// Persistent batched launches (gpp_batched.cu): a work queue of tiles over
// many states.  kind 0 = occupied-band tile (band_tile is the band), 1 =
// unoccupied-band tile; `tile` is the absolute slot in the state's achtemp
// partial segment.
struct BatchItem {
    int state, kind, row_tile, band_tile, iw_chunk, tile;
};

// Pipeline variant of the mixed kernel chosen for (device, nw).
int tuned_mixed_variant(int dev, int nw);

// Argument checks shared by every entry point (gpp_api.cu): sizes, pointers,
// enum values and size overflow; on failure they record the message for
// gpp_last_error_message.
gpp_status validate(const gpp_problem *problem);
Problem to_problem(const gpp_problem &q);
// Grid limits of one call's launches (occupied bands, unoccupied band tiles,
// frequency chunks), GPP_ERR_UNSUPPORTED beyond them.
gpp_status check_grid_limits(const Problem &p, int occupied_bands, int unoccupied_bands,
                             const TileShape &ns, bool gemm);

// Per-thread launch counter (gpp_launch_count).
void count_launch(int n = 1);

// The largest shared-memory carve-out for a kernel that runs beside the
// tensor-core GEMM (one block of ~193 KB of shared memory per SM): an SM
// changes its L1/shared split only when no block is resident, so blocks that
// left it at a small split keep the GEMM's blocks off that SM until they
// drain.  A hint: a refusal is cleared and ignored.
template <typename Kernel>
inline void prefer_max_shared(Kernel *kernel) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        cudaGetLastError();
}

}  // namespace gpp

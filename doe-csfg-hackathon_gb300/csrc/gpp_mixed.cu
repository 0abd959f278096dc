// gpp_mixed.cu -- mixed-precision unoccupied-band kernel (placeholder until
// the float-float kernel lands).
#include "gpp_kernels.h"

namespace gpp {
size_t mixed_split_bytes(const Problem &) { return 0; }
TileShape mixed_noflag_shape(const Problem &p) { return fp64_noflag_shape(p); }
cudaError_t launch_mixed_noflag(const Problem &, const Partials &, void *, int, int, cudaStream_t) {
    return cudaErrorNotSupported;
}
}  // namespace gpp

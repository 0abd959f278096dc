/* Force-included when compiling the reference's gppCuda.cu for its device
 * code (oracle/build_oracle.py): CUDA 13 replaced
 * cudaMemPrefetchAsync(ptr, bytes, int device, stream) by a form taking a
 * cudaMemLocation and flags, and gppCuda.cu calls the old one
 * (gppCuda.cu:356-362).  This overload of the old form lets the source
 * compile unchanged; only the device code is kept. */
#pragma once
#include <cuda_runtime_api.h>

static inline cudaError_t cudaMemPrefetchAsync(const void *ptr, size_t bytes, int device,
                                               cudaStream_t stream = 0) {
    cudaMemLocation loc;
    loc.type = cudaMemLocationTypeDevice;
    loc.id = device;
    return cudaMemPrefetchAsync(ptr, bytes, loc, 0, stream);
}

// gpp_static.cu -- gpp_sigma_static_scratch: the FP64 GPP sigma reduction
// for callers that cannot allocate device memory.
//
// Who needs it: host codes that hand the whole GPU to their own memory arena
// or to another runtime before calling in (so cudaMalloc would fail or steal
// memory they have budgeted), and codes that must not pay cudaMalloc's
// implicit device-wide synchronisation in the middle of a time step.
// gpp_sigma draws its block-partial workspace from the stream-ordered pool;
// this entry point instead keeps that scratch in a fixed array in the
// library's own device image, so it performs no allocation of any kind.
//
// Limits and sharing rules:
//  * the scratch array is kStaticScratchBytes (8 MiB) and is resident on
//    every GPU that loads the library, for the life of the process;
//  * a problem whose block partials need more than that is rejected with
//    GPP_ERR_UNSUPPORTED before anything is launched (the production shape,
//    512 bands x 1638 rows x 3 frequencies, needs ~5 MiB);
//  * all calls share the one array: calls whose GPU work overlaps in time
//    (different streams, different host threads) race on it and corrupt each
//    other's results -- serialise them on one stream.  Every slot is written
//    before it is read, so contents left by a previous call are harmless;
//  * FP64 only, outputs achtemp and asxtemp only (acht_n1_loc and achstemp
//    must be NULL); rows whose inv_igp_index / indinv is invalid contribute
//    nothing, as in gpp_sigma, but are not reported by gpp_wait;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture begins.
#include <mutex>

#include <cstdio>

#include "gpp_gb300.h"
#include "gpp_kernels.h"

namespace gpp {

// Defined with the rest of the error plumbing in gpp_api.cu.
gpp_status set_error(gpp_status s, const char *msg);

namespace {

constexpr size_t kStaticScratchBytes = size_t(8) << 20;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
// Sink for the kernels' index-fault bits (never read back).
static __device__ int g_static_fault;

std::mutex g_static_mutex;
void *g_static_scratch_addr[256] = {};
int *g_static_fault_addr[256] = {};

// Device addresses of the two arrays for the current device (looked up once).
gpp_status static_addresses(void **scratch, int **fault) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= 256) return set_error(GPP_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_static_mutex);
    if (!g_static_scratch_addr[dev]) {
        void *s = nullptr;
        void *f = nullptr;
        e = cudaGetSymbolAddress(&s, g_static_scratch);
        if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
        e = cudaGetSymbolAddress(&f, g_static_fault);
        if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
        g_static_scratch_addr[dev] = s;
        g_static_fault_addr[dev] = static_cast<int *>(f);
    }
    *scratch = g_static_scratch_addr[dev];
    *fault = g_static_fault_addr[dev];
    return GPP_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace gpp

using namespace gpp;

extern "C" gpp_status gpp_sigma_static_scratch(const gpp_problem *problem, const gpp_outputs *out,
                                               gpp_stream_t stream) {
    if (!out) return set_error(GPP_ERR_INVALID_ARGUMENT, "outputs is NULL");
    // The same argument checks as gpp_sigma: sizes, pointers, enum values,
    // size overflow.
    gpp_status st = validate(problem);
    if (st != GPP_OK) return st;
    if (problem->precision != GPP_PRECISION_FP64)
        return set_error(GPP_ERR_UNSUPPORTED, "gpp_sigma_static_scratch computes in FP64 only");
    if (!out->achtemp || !out->asxtemp)
        return set_error(GPP_ERR_INVALID_ARGUMENT, "outputs achtemp/asxtemp are required");
    if (out->acht_n1_loc || out->achstemp)
        return set_error(GPP_ERR_UNSUPPORTED,
                         "gpp_sigma_static_scratch returns achtemp and asxtemp only");
    const Problem p = to_problem(*problem);

    // Block-partial layout, as gpp_sigma uses it: achtemp partials of the
    // occupied then unoccupied blocks, then asxtemp partials.
    const bool has_flag = p.nv > 0 && p.ng > 0;
    const bool has_noflag = p.nb > p.nv && p.ng > 0;
    const TileShape fs = flag_shape(p), ns = fp64_noflag_shape(p);
    const long long tiles_f = has_flag ? (long long)ceil_div(p.ng, fs.rg) * p.nv : 0;
    const long long tiles_n =
        has_noflag ? (long long)ceil_div(p.ng, ns.rg) * ceil_div(p.nb - p.nv, ns.rn) : 0;
    // The grid limits of gpp_sigma's launches (this entry point never takes
    // the band-sum GEMM path).
    st = check_grid_limits(p, has_flag ? p.nv : 0, has_noflag ? p.nb - p.nv : 0, ns, false);
    if (st != GPP_OK) return st;
    const size_t ach_bytes = align256(sizeof(double2) * (size_t)((tiles_f + tiles_n) * p.nw));
    const size_t need = ach_bytes + align256(sizeof(double2) * (size_t)(tiles_f * p.nw));
    if (need > kStaticScratchBytes) {
        char msg[200];
        snprintf(msg, sizeof(msg),
                 "problem needs %zu bytes of block-partial scratch; the static buffer holds %zu",
                 need, kStaticScratchBytes);
        return set_error(GPP_ERR_UNSUPPORTED, msg);
    }

    void *scratch = nullptr;
    int *fault = nullptr;
    st = static_addresses(&scratch, &fault);
    if (st != GPP_OK) return st;

    Partials part{};
    part.ach = static_cast<double2 *>(scratch);
    part.ach_seg = tiles_f + tiles_n;
    part.asx = reinterpret_cast<double2 *>(static_cast<char *>(scratch) + ach_bytes);
    part.asx_seg = tiles_f;
    part.n1 = nullptr;
    part.n1_seg = 0;
    part.err = fault;

    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (has_flag) {
        part.ach_tile0 = 0;
        e = launch_flag_fp64(p, part, s);
    }
    if (e == cudaSuccess && has_noflag) {
        part.ach_tile0 = (int)tiles_f;
        e = launch_noflag_fp64(p, part, p.nv, p.nb, s);
    }
    if (e == cudaSuccess) {
        ReduceOut ro{reinterpret_cast<double2 *>(out->achtemp), nullptr, nullptr, 0};
        e = launch_reduce(part.ach, part.ach_seg, (int)part.ach_seg, p.nw, ro, s);
    }
    if (e == cudaSuccess) {
        ReduceOut ro{reinterpret_cast<double2 *>(out->asxtemp), nullptr, nullptr, 0};
        e = launch_reduce(part.asx, part.asx_seg, (int)part.asx_seg, p.nw, ro, s);
    }
    if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
    return GPP_OK;
}

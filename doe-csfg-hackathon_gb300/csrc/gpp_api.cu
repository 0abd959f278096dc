// gpp_api.cu -- the C ABI of libgpp_gb300.so (include/gpp_gb300.h): argument
// validation, workspace, kernel dispatch, the deterministic reduction plan,
// streams, error reporting and the host-buffer (end-to-end) path.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include <algorithm>
#include <chrono>
#include <cstdlib>

#include "gpp_gb300.h"
#include "gpp_gemm.h"
#include "gpp_gemm_mixed.h"
#include "gpp_kernels.h"

namespace gpp {

namespace {
thread_local std::string t_err;
thread_local unsigned long long t_launches = 0;
thread_local cudaStream_t t_compat_stream = nullptr;
thread_local int t_dropin_precision = -1;  // -1: the process default
thread_local int t_gemm_path = -1;         // -1: automatic, 0: never, 1: whenever it applies,
                                            // 2: as 1 with the FP64 GEMM on the FP64 pipe
thread_local bool t_timing = false;
thread_local cudaEvent_t t_ev0 = nullptr, t_ev1 = nullptr;
thread_local bool t_timed = false;
}  // namespace

void count_launch(int n) { t_launches += (unsigned long long)n; }

bool fp64_gemm_on_tensor_cores() { return t_gemm_path != 2; }

// Records `msg` as this thread's gpp_last_error_message and returns `s`.
gpp_status set_error(gpp_status s, const char *msg) {
    t_err = msg ? msg : "";
    return s;
}

namespace {

gpp_status fail(gpp_status s, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_err = buf;
    return s;
}

gpp_status cuda_fail(cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(GPP_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(GPP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define GPP_CUDA_TRY(call, what)                          \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

// One persistent fault word and one workspace pool per device (created on
// first use).  The pool is the library's own: workspace allocations stay
// cached between calls (release threshold: never), and the caller's
// default pool and its settings are left untouched.
std::mutex g_dev_mutex;
int *g_err_word[256] = {};
cudaMemPool_t g_pool[256] = {};

gpp_status device_setup(int *dev_out, int **err_out, cudaMemPool_t *pool_out = nullptr) {
    int dev = 0;
    GPP_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 256) return fail(GPP_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lk(g_dev_mutex);
    if (!g_err_word[dev]) {
        int *w = nullptr;
        GPP_CUDA_TRY(cudaMalloc(&w, sizeof(int)), "cudaMalloc(fault word)");
        GPP_CUDA_TRY(cudaMemset(w, 0, sizeof(int)), "cudaMemset(fault word)");
        g_err_word[dev] = w;
    }
    if (!g_pool[dev]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        GPP_CUDA_TRY(cudaMemPoolCreate(&pool, &props), "cudaMemPoolCreate(workspace pool)");
        unsigned long long thr = ~0ull;
        cudaError_t e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(pool);
            return cuda_fail(e, "cudaMemPoolSetAttribute(workspace pool)");
        }
        g_pool[dev] = pool;
    }
    *dev_out = dev;
    *err_out = g_err_word[dev];
    if (pool_out) *pool_out = g_pool[dev];
    return GPP_OK;
}

// Stream-ordered workspace from the library's pool of the current device.
gpp_status workspace_alloc(void **ptr, size_t bytes, cudaStream_t s) {
    int dev = 0;
    int *err = nullptr;
    cudaMemPool_t pool = nullptr;
    gpp_status st = device_setup(&dev, &err, &pool);
    if (st != GPP_OK) return st;
    GPP_CUDA_TRY(cudaMallocFromPoolAsync(ptr, bytes, pool, s), "cudaMallocFromPoolAsync(workspace)");
    return GPP_OK;
}

// Where the final fixed-order sums go.
struct OutSpec {
    double2 *ach = nullptr;  // [nw] complex (overwrite or accumulate)
    double *ach_re = nullptr, *ach_im = nullptr;  // split, accumulate
    double2 *asx = nullptr;  // [nw]
    double2 *n1 = nullptr;   // [nb] indexed by absolute band
    double2 *achs = nullptr; // [1]
    double *achs_re = nullptr, *achs_im = nullptr;
    int accumulate = 0;
};

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Pipeline variant of the mixed kernel per (device, frequency chunk): chosen
// by gpp_autotune or gpp_set_variant, else the compiled-in default.  A
// thread-local override lets the autotuner time each variant.
std::mutex g_tune_mutex;
int g_tuned[256][9];  // [device][nwc 1..8]; 0 = unset, else variant + 1
bool g_tune_loaded = false;
thread_local int t_force_variant = -1;

int nwc_of(int nw) { return nw <= 4 ? nw : 8; }

void tune_cache_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = getenv("GPP_TUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    int dev, nwc, v;
    while (fscanf(f, "%d %d %d", &dev, &nwc, &v) == 3)
        if (dev >= 0 && dev < 256 && nwc >= 1 && nwc <= 8 && v >= 0 && v < mixed_variant_count())
            g_tuned[dev][nwc] = v + 1;
    fclose(f);
}

void tune_cache_save_locked() {
    const char *path = getenv("GPP_TUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "w");
    if (!f) return;
    for (int d = 0; d < 256; ++d)
        for (int n = 1; n <= 8; ++n)
            if (g_tuned[d][n]) fprintf(f, "%d %d %d\n", d, n, g_tuned[d][n] - 1);
    fclose(f);
}

int mixed_variant_for(int dev, int nw) {
    if (t_force_variant >= 0 && mixed_variant_valid(t_force_variant, nw)) return t_force_variant;
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    tune_cache_load_locked();
    const int v = g_tuned[dev & 255][nwc_of(nw)];
    return (v && mixed_variant_valid(v - 1, nw)) ? v - 1 : mixed_default_variant();
}

// Per host thread and device: a highest-priority side stream plus fork/join
// events.  The mixed path runs the FP64 occupied-band kernel there, beside the
// FP32 unoccupied-band kernel: the two keep different pipes busy on the same
// SMs.  Fork and join are stream-ordered, so the pair is also captured
// correctly into a CUDA graph.
struct SideStream {
    int dev = -1;
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
thread_local SideStream t_side;

// Precision of the drop-in entry points: gpp_set_dropin_precision on this
// thread, else GPP_DROPIN_PRECISION=mixed|fp64 in the environment, else FP64.
int dropin_precision() {
    if (t_dropin_precision >= 0) return t_dropin_precision;
    static const int env = [] {
        const char *v = getenv("GPP_DROPIN_PRECISION");
        return (v && strcmp(v, "mixed") == 0) ? (int)GPP_PRECISION_MIXED : (int)GPP_PRECISION_FP64;
    }();
    return env;
}

// Whether the unoccupied bands of a call with band-independent wx go through
// the band-sum GEMM (FP64: gpp_gemm.cu, mixed: gpp_gemm_mixed.cu):
// automatically from 32 unoccupied bands on (below that the per-term kernel
// is as fast), or as gpp_set_gemm_path forces.
constexpr int kGemmMinBands = 32;
bool gemm_path(int wx_stride, int bands) {
    if (wx_stride != 0 || bands <= 0) return false;
    return t_gemm_path < 0 ? bands >= kGemmMinBands : t_gemm_path >= 1;
}

// Whether the mixed path runs the occupied-band kernel concurrently on the
// side stream (GPP_OVERLAP_OCCUPIED=1) or before the unoccupied-band kernel
// on the caller's stream (default).  Measured on GB300 at the production
// shape, the concurrent form was slower: the FP64 blocks take register and
// warp slots the issue-bound FP32 kernel needs.
bool overlap_occupied() {
    static const bool on = [] {
        const char *v = getenv("GPP_OVERLAP_OCCUPIED");
        return v && v[0] == '1';
    }();
    return on;
}

// Whether calls whose band sum runs on the tensor cores run the
// occupied-band kernel concurrently on the side stream (the default), so
// that the FP64 / FP32 pipes and the tensor cores work at the same time;
// GPP_OVERLAP_TENSOR_GEMM=0 runs it first on the caller's stream.  Read on
// every call.
bool overlap_tensor_gemm() {
    const char *v = getenv("GPP_OVERLAP_TENSOR_GEMM");
    return !(v && v[0] == '0');
}

gpp_status side_stream(int dev, SideStream **out) {
    if (t_side.dev != dev) {
        int lo = 0, hi = 0;
        GPP_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi), "cudaDeviceGetStreamPriorityRange");
        SideStream n;
        GPP_CUDA_TRY(cudaStreamCreateWithPriority(&n.st, cudaStreamNonBlocking, hi),
                     "cudaStreamCreateWithPriority");
        GPP_CUDA_TRY(cudaEventCreateWithFlags(&n.fork, cudaEventDisableTiming), "cudaEventCreate");
        GPP_CUDA_TRY(cudaEventCreateWithFlags(&n.join, cudaEventDisableTiming), "cudaEventCreate");
        n.dev = dev;
        t_side = n;  // a stream of a previously used device is kept alive
    }
    *out = &t_side;
    return GPP_OK;
}

// Runs the bands [b0, b1) of problem p: occupied bands (< nv) through the
// flag kernel, the rest through the FP64 or mixed unoccupied kernel, then
// reduces all block partials in a fixed order into the outputs.
// Row pieces of a call whose G' rows arrive on the device in parts (the
// host path): piece k covers row pairs [pair[k], pair[k+1]) and its kernels
// start once ready[k] has fired.  The partial sums land in the same slots
// as one launch over all rows, so the result does not depend on the pieces.
constexpr int kMaxRowPieces = 16;
struct RowPieces {
    int n = 0;
    int pair[kMaxRowPieces + 1] = {};
    cudaEvent_t ready[kMaxRowPieces] = {};
    cudaEvent_t started[kMaxRowPieces] = {};  // optional: compute stream passed ready[k]
};

gpp_status run_sigma(const Problem &p, int b0, int b1, int precision, const OutSpec &o,
                     bool do_main, cudaStream_t s, const RowPieces *pieces = nullptr) {
    int dev = 0;
    int *err = nullptr;
    gpp_status st = device_setup(&dev, &err);
    if (st != GPP_OK) return st;

    const int fb0 = b0, fb1 = do_main ? (b1 < p.nv ? b1 : p.nv) : b0;
    const int nb0 = do_main ? (b0 > p.nv ? b0 : p.nv) : b1, nb1 = b1;
    const bool has_flag = fb1 > fb0 && p.ng > 0;
    const bool has_noflag = nb1 > nb0 && p.ng > 0;
    const bool mixed = precision == GPP_PRECISION_MIXED && (has_noflag || has_flag);

    const TileShape fs = flag_shape(p);  // same tiling for the FP64 and the mixed occupied tile
    const int variant = mixed ? mixed_variant_for(dev, p.nw) : 0;
    const TileShape ns = mixed ? mixed_noflag_shape(p, variant) : fp64_noflag_shape(p);
    const bool want_n1 = o.n1 && p.nw >= 3 && p.ng > 0;
    const bool gemm = has_noflag && gemm_path(p.wx_stride, nb1 - nb0);
    const long long rows_f = has_flag ? ceil_div(p.ng, fs.rg) : 0;
    const long long rows_n = has_noflag ? ceil_div(p.ng, ns.rg) : 0;
    const long long tiles_f = has_flag ? rows_f * (fb1 - fb0) : 0;
    // The GEMM path writes one partial per row tile (all bands at once).
    const long long tiles_n =
        !has_noflag ? 0 : gemm ? rows_n : rows_n * ceil_div(nb1 - nb0, ns.rn);
    st = check_grid_limits(p, has_flag ? fb1 - fb0 : 0, has_noflag ? nb1 - nb0 : 0, ns, gemm);
    if (st != GPP_OK) return st;
    if (has_flag && fb0 != 0)
        return fail(GPP_ERR_UNSUPPORTED, "occupied-band launches start at band 0");
    const long long ach_seg = tiles_f + tiles_n;
    const long long n1_seg = rows_f > rows_n ? rows_f : rows_n;
    const bool want_achs = (o.achs || o.achs_re) && p.ng > 0 && b1 > b0;
    const int achs_blocks = want_achs ? achstemp_blocks(p) : 0;

    size_t off = 0;
    const size_t o_ach = off; off = align_up(off + sizeof(double2) * (size_t)(ach_seg * p.nw));
    const size_t o_asx = off; off = align_up(off + sizeof(double2) * (size_t)(tiles_f * p.nw));
    const size_t o_n1 = off; off = align_up(off + (want_n1 ? sizeof(double2) * (size_t)(n1_seg * p.nb) : 0));
    const size_t o_st = off; off = align_up(off + sizeof(double2) * (size_t)achs_blocks);
    const size_t o_next = off; off = align_up(off + sizeof(int));  // work counter
    const size_t o_split = off; off = align_up(off + (mixed ? mixed_split_bytes(p) : 0));
    // Band sums on the tensor cores (both precisions; mixed precision then
    // splits G into its float-float planes) unless gpp_set_gemm_path(2).
    const bool tensor = gemm && fp64_gemm_on_tensor_cores();
    const size_t gemm_ws = !gemm ? 0 : mixed ? mixed_gemm_bytes(p, nb1 - nb0, want_n1 && !tensor)
                                            : gemm_bytes(p, nb1 - nb0, want_n1);
    const size_t o_gemm = off; off = align_up(off + gemm_ws);
    const size_t o_gemm64 = off;
    off = align_up(off + (mixed && tensor ? gemm_bytes(p, nb1 - nb0, want_n1) : 0));
    const size_t ws_bytes = off > 0 ? off : 256;

    void *ws = nullptr;
    st = workspace_alloc(&ws, ws_bytes, s);
    if (st != GPP_OK) return st;
    char *w = static_cast<char *>(ws);

    Partials part{};
    part.ach = reinterpret_cast<double2 *>(w + o_ach);
    part.ach_seg = ach_seg;
    part.asx = reinterpret_cast<double2 *>(w + o_asx);
    part.asx_seg = tiles_f;
    part.n1 = want_n1 ? reinterpret_cast<double2 *>(w + o_n1) : nullptr;
    part.n1_seg = (int)n1_seg;
    part.err = err;

    cudaError_t e = cudaSuccess;
    if (want_n1 && (rows_f != rows_n) && has_flag && has_noflag) {
        // Different row tilings: pad the shorter per-band segments with zeros.
        e = cudaMemsetAsync(part.n1, 0, sizeof(double2) * (size_t)(n1_seg * p.nb), s);
    }
    if (e == cudaSuccess && mixed)  // float-float planes of every band the call touches
        e = launch_split_bands(p, w + o_split, has_flag ? fb0 : nb0, has_noflag ? nb1 : fb1, s);
    SideStream *side = nullptr;
    const bool overlap =
        has_flag && has_noflag && !pieces &&
        (gemm && tensor ? overlap_tensor_gemm() : mixed && overlap_occupied());
    // FP64 with the per-band output: the occupied-band kernel starts once the
    // tensor-core band sum's slicing passes are queued rather than with them
    // (measured 28.0 -> 26.5 ms per production call; without the per-band
    // output it made calls queued back to back slower, 22.7 -> 25.7 ms).
    const bool late_fork = overlap && gemm && tensor && !mixed && want_n1;
    RowPieces whole;
    whole.n = 1;
    whole.pair[0] = 0;
    whole.pair[1] = (p.ng + 1) / 2;
    const RowPieces &pc = pieces ? *pieces : whole;
    if (overlap) {
        st = side_stream(dev, &side);
        if (st != GPP_OK) {
            cudaFreeAsync(ws, s);
            return st;
        }
    }
    for (int k = 0; k < pc.n && e == cudaSuccess; ++k) {
        RowTiles rt;
        rt.begin = pc.pair[k];
        rt.end = pc.pair[k + 1];
        if (pieces) e = cudaStreamWaitEvent(s, pc.ready[k], 0);
        if (e == cudaSuccess && pieces && pc.started[k]) e = cudaEventRecord(pc.started[k], s);
        if (e == cudaSuccess && mixed) e = launch_split_rows(p, w + o_split, rt, s);
        if (e == cudaSuccess && overlap && !late_fork)
            e = cudaEventRecord(side->fork, s);  // planes written
        if (e == cudaSuccess && has_flag && !overlap) {
            part.ach_tile0 = 0;
            e = mixed ? launch_flag_mixed(p, part, w + o_split, s, rt)
                      : launch_flag_fp64(p, part, s, rt);
        }
        if (e == cudaSuccess && has_noflag) {
            part.ach_tile0 = (int)tiles_f;
            if (k == 0 && t_timing && t_ev0) cudaEventRecord(t_ev0, s);
            if (gemm && mixed) {
                st = GPP_OK;
                if (k == 0 && tensor) {
                    st = gemm_band_sum(p, part, w + o_gemm64, nb0, nb1, s);
                    if (st == GPP_OK)
                        st = mixed_gemm_planes_from(
                            p, w + o_gemm, nb0, nb1,
                            gemm_g(p, w + o_gemm64, nb1 - nb0, want_n1), s);
                } else if (k == 0) {
                    st = mixed_gemm_band_sum(p, part, w + o_split, w + o_gemm, nb0, nb1, s);
                }
                if (st == GPP_OK)
                    st = mixed_gemm_rows(p, part, w + o_split, w + o_gemm, nb0, nb1, s, rt);
                if (st == GPP_OK && k == pc.n - 1)
                    st = tensor ? gemm_per_band(p, part, w + o_gemm64, nb0, nb1, s, w + o_split)
                                : mixed_gemm_per_band(p, part, w + o_split, w + o_gemm, nb0, nb1, s);
                if (st != GPP_OK) {
                    cudaFreeAsync(ws, s);
                    return st;
                }
            } else if (gemm) {
                st = GPP_OK;
                if (k == 0)
                    st = gemm_band_sum(p, part, w + o_gemm, nb0, nb1, s,
                                       late_fork ? side->fork : nullptr);
                if (st == GPP_OK) st = gemm_rows(p, part, w + o_gemm, nb0, nb1, s, rt);
                if (st == GPP_OK && k == pc.n - 1) st = gemm_per_band(p, part, w + o_gemm, nb0, nb1, s);
                if (st != GPP_OK) {
                    cudaFreeAsync(ws, s);
                    return st;
                }
            } else {
                e = mixed ? launch_mixed_noflag(p, part, w + o_split, nb0, nb1, s, variant, rt)
                          : launch_noflag_fp64(p, part, nb0, nb1, s, rt);
            }
            if (k == pc.n - 1 && t_timing && t_ev1) {
                cudaEventRecord(t_ev1, s);
                t_timed = true;
            }
        }
    }
    if (e == cudaSuccess && overlap) {
        e = cudaStreamWaitEvent(side->st, side->fork, 0);
        part.ach_tile0 = 0;
        if (e == cudaSuccess)
            // FP64 beside the tensor-core GEMM: one persistent block per SM
            // taking row tiles from a counter.  The GEMM's MMAs slow down under
            // any co-resident load and stop while FP64 instructions are in
            // flight on their SM, so a lighter load leaves them more time.  The
            // float-float kernel keeps its grid (three blocks per SM carry its
            // FP32 work; one was slower).
            e = mixed ? launch_flag_mixed(p, part, w + o_split, side->st, RowTiles(), 0,
                                          reinterpret_cast<int *>(w + o_next))
                      : launch_flag_fp64(p, part, side->st, RowTiles(), gemm && tensor ? 1 : 0,
                                         reinterpret_cast<int *>(w + o_next));
        if (e == cudaSuccess) e = cudaEventRecord(side->join, side->st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, side->join, 0);
    }
    if (e == cudaSuccess && want_achs)
        e = launch_achstemp(p, reinterpret_cast<double2 *>(w + o_st), err, s);

    // Fixed-order reduction of the block partials.
    if (e == cudaSuccess && (o.ach || o.ach_re)) {
        ReduceOut ro{o.ach, o.ach_re, o.ach_im, o.accumulate};
        e = launch_reduce(part.ach, ach_seg, (int)ach_seg, p.nw, ro, s);
    }
    if (e == cudaSuccess && o.asx) {
        ReduceOut ro{o.asx, nullptr, nullptr, o.accumulate};
        e = launch_reduce(part.asx, tiles_f, (int)tiles_f, p.nw, ro, s);
    }
    if (e == cudaSuccess && want_n1 && b1 > b0) {
        ReduceOut ro{o.n1 + b0, nullptr, nullptr, o.accumulate};
        e = launch_reduce(part.n1 + (size_t)b0 * n1_seg, n1_seg, (int)n1_seg, b1 - b0, ro, s);
    }
    if (e == cudaSuccess && want_achs) {
        ReduceOut ro{o.achs, o.achs_re, o.achs_im, o.accumulate};
        e = launch_reduce(reinterpret_cast<double2 *>(w + o_st), achs_blocks, achs_blocks, 1, ro, s);
    }
    cudaError_t e2 = cudaFreeAsync(ws, s);
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeAsync(workspace)");
    return GPP_OK;
}

}  // namespace

static bool mul_ok(long long a, long long b, long long lim) { return a == 0 || b <= lim / a; }

gpp_status validate(const gpp_problem *pr) {
    if (!pr) return fail(GPP_ERR_INVALID_ARGUMENT, "problem is NULL");
    const gpp_problem &p = *pr;
    if (p.number_bands < 0 || p.nvband < 0 || p.nvband > p.number_bands)
        return fail(GPP_ERR_INVALID_ARGUMENT, "need 0 <= nvband <= number_bands (got %d, %d)",
                    p.nvband, p.number_bands);
    if (p.ncouls <= 0) return fail(GPP_ERR_INVALID_ARGUMENT, "ncouls must be > 0 (got %d)", p.ncouls);
    if (p.ngpown < 0) return fail(GPP_ERR_INVALID_ARGUMENT, "ngpown must be >= 0 (got %d)", p.ngpown);
    if (p.nw <= 0) return fail(GPP_ERR_INVALID_ARGUMENT, "nw must be > 0 (got %d)", p.nw);
    if (p.wx_stride != 0 && p.wx_stride < p.nw)
        return fail(GPP_ERR_INVALID_ARGUMENT, "wx_stride must be 0 or >= nw (got %d)", p.wx_stride);
    if (p.semantics != GPP_SEM_COMPLEX_SEQ && p.semantics != GPP_SEM_KERSEQ)
        return fail(GPP_ERR_INVALID_ARGUMENT, "unknown semantics %d", p.semantics);
    if (p.precision != GPP_PRECISION_FP64 && p.precision != GPP_PRECISION_MIXED)
        return fail(GPP_ERR_INVALID_ARGUMENT, "unknown precision %d", p.precision);
    const long long lim = (long long)1 << 60;
    if (!mul_ok(p.number_bands, p.ncouls, lim) || !mul_ok(p.ngpown, p.ncouls, lim) ||
        !mul_ok((long long)p.number_bands * (p.wx_stride ? 1 : 0), p.wx_stride ? p.wx_stride : 1, lim))
        return fail(GPP_ERR_INVALID_ARGUMENT, "array sizes overflow");
    if (p.number_bands > 0 && (!p.aqsmtemp || !p.aqsntemp))
        return fail(GPP_ERR_INVALID_ARGUMENT, "aqsmtemp/aqsntemp is NULL");
    if (p.ngpown > 0 && (!p.I_eps_array || !p.wtilde_array || !p.inv_igp_index))
        return fail(GPP_ERR_INVALID_ARGUMENT, "I_eps_array/wtilde_array/inv_igp_index is NULL");
    if (!p.vcoul || !p.wx_array) return fail(GPP_ERR_INVALID_ARGUMENT, "vcoul/wx_array is NULL");
    return GPP_OK;
}

Problem to_problem(const gpp_problem &q) {
    Problem p;
    p.aqsm = reinterpret_cast<const double2 *>(q.aqsmtemp);
    p.aqsn = reinterpret_cast<const double2 *>(q.aqsntemp);
    p.ieps = reinterpret_cast<const double2 *>(q.I_eps_array);
    p.wt = reinterpret_cast<const double2 *>(q.wtilde_array);
    p.vcoul = q.vcoul;
    p.inv_igp = q.inv_igp_index;
    p.indinv = q.indinv;
    p.wx = q.wx_array;
    p.wx_stride = q.wx_stride;
    p.nb = q.number_bands;
    p.nv = q.nvband;
    p.nc = q.ncouls;
    p.ng = q.ngpown;
    p.nw = q.nw;
    p.occ = q.occ;
    p.semantics = q.semantics;
    return p;
}

// Grid limits of one call's launches: the unoccupied-band kernels' grid.x
// counts (row tile, band tile) pairs (<= 2^31 - 1) and their band tiles are
// kept <= 65535; grid.y of the occupied-band kernels counts occupied bands,
// and frequency chunks stay <= 65535.
gpp_status check_grid_limits(const Problem &p, int occupied_bands, int unoccupied_bands,
                             const TileShape &ns, bool gemm) {
    if (unoccupied_bands > 0 && !gemm && ceil_div(unoccupied_bands, ns.rn) > 65535)
        return fail(GPP_ERR_UNSUPPORTED, "too many bands for one launch (%d)", unoccupied_bands);
    // The per-term kernels walk (row tile, band tile) pairs along grid.x.
    if (unoccupied_bands > 0 && !gemm &&
        (long long)ceil_div(p.ng, ns.rg) * ceil_div(unoccupied_bands, ns.rn) > 2147483647LL)
        return fail(GPP_ERR_UNSUPPORTED, "too many tiles for one launch");
    if (ceil_div(p.nw, ns.nwc) > 65535 || occupied_bands > 65535)
        return fail(GPP_ERR_UNSUPPORTED, "too many frequencies or occupied bands");
    return GPP_OK;
}

int tuned_mixed_variant(int dev, int nw) { return mixed_variant_for(dev, nw); }

}  // namespace gpp

using namespace gpp;

extern "C" {

// The current device's fault word (used by the batch planner), or NULL.
int *gpp_internal_fault_word(void) {
    int dev = 0;
    int *err = nullptr;
    return device_setup(&dev, &err) == GPP_OK ? err : nullptr;
}

const char *gpp_last_error_message(void) { return t_err.c_str(); }
unsigned long long gpp_launch_count(void) { return t_launches; }
void gpp_reset_launch_count(void) { t_launches = 0; }

gpp_status gpp_set_stream(gpp_stream_t stream) {
    t_compat_stream = reinterpret_cast<cudaStream_t>(stream);
    return GPP_OK;
}
gpp_stream_t gpp_get_stream(void) { return reinterpret_cast<gpp_stream_t>(t_compat_stream); }

gpp_status gpp_set_gemm_path(int mode) {
    if (mode < -1 || mode > 2) return fail(GPP_ERR_INVALID_ARGUMENT, "gemm path mode %d", mode);
    t_gemm_path = mode;
    return GPP_OK;
}

gpp_status gpp_set_dropin_precision(int precision) {
    if (precision != -1 && precision != GPP_PRECISION_FP64 && precision != GPP_PRECISION_MIXED)
        return fail(GPP_ERR_INVALID_ARGUMENT, "unknown precision %d", precision);
    t_dropin_precision = precision;
    return GPP_OK;
}
int gpp_get_dropin_precision(void) { return dropin_precision(); }

}  // extern "C"

namespace {
// gpp_sigma, optionally over G' rows that reach the device in pieces.
gpp_status sigma_impl(const gpp_problem *problem, const gpp_outputs *out, cudaStream_t s,
                      const RowPieces *pieces) {
    gpp_status st = validate(problem);
    if (st != GPP_OK) return st;
    if (!out || !out->achtemp || !out->asxtemp)
        return fail(GPP_ERR_INVALID_ARGUMENT, "outputs achtemp/asxtemp are required");
    if (out->acht_n1_loc && problem->nw < 3)
        return fail(GPP_ERR_INVALID_ARGUMENT, "acht_n1_loc needs nw >= 3 (it sums the iw = 2 column)");
    Problem p = to_problem(*problem);
    OutSpec o;
    o.ach = reinterpret_cast<double2 *>(out->achtemp);
    o.asx = reinterpret_cast<double2 *>(out->asxtemp);
    o.n1 = reinterpret_cast<double2 *>(out->acht_n1_loc);
    o.achs = reinterpret_cast<double2 *>(out->achstemp);
    o.accumulate = 0;
    if (o.n1 && (p.nb == 0 || p.ng == 0)) {
        cudaError_t e = cudaMemsetAsync(o.n1, 0, sizeof(double2) * (size_t)p.nb, s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(acht_n1_loc)");
    }
    if (o.achs && (p.nb == 0 || p.ng == 0)) {
        cudaError_t e = cudaMemsetAsync(o.achs, 0, sizeof(double2), s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(achstemp)");
    }
    return run_sigma(p, 0, p.nb, problem->precision, o, true, s, pieces);
}
}  // namespace

extern "C" {

gpp_status gpp_sigma(const gpp_problem *problem, const gpp_outputs *out, gpp_stream_t stream) {
    return sigma_impl(problem, out, reinterpret_cast<cudaStream_t>(stream), nullptr);
}

gpp_status gpp_kernel_gpu(const gpp_complex *wtilde_array, const gpp_complex *aqsntemp,
                          const gpp_complex *aqsmtemp, const gpp_complex *I_eps_array, int ncouls,
                          int ngpown, int number_bands, const double *wx_array, double *achtemp_re,
                          double *achtemp_im, const double *vcoul, int nstart, int nend,
                          const int *indinv, const int *inv_igp_index) {
    gpp_problem q{};
    q.number_bands = number_bands;
    q.nvband = 0;
    q.ncouls = ncouls;
    q.ngpown = ngpown;
    q.nw = nend - nstart;
    q.aqsmtemp = aqsmtemp;
    q.aqsntemp = aqsntemp;
    q.I_eps_array = I_eps_array;
    q.wtilde_array = wtilde_array;
    q.vcoul = vcoul;
    q.inv_igp_index = inv_igp_index;
    q.indinv = indinv;
    q.wx_array = wx_array;
    q.wx_stride = 0;
    q.occ = 1.0;
    q.semantics = GPP_SEM_COMPLEX_SEQ;
    q.precision = dropin_precision();
    gpp_status st = validate(&q);
    if (st != GPP_OK) return st;
    if (!achtemp_re || !achtemp_im) return fail(GPP_ERR_INVALID_ARGUMENT, "achtemp_re/im is NULL");
    OutSpec o;
    o.ach_re = achtemp_re;
    o.ach_im = achtemp_im;
    o.accumulate = 1;
    return run_sigma(to_problem(q), 0, number_bands, q.precision, o, true, t_compat_stream);
}

static gpp_problem compat_problem(int number_bands, int nvband, int ngpown, int ncouls,
                                  const int *inv_igp_index, const double *wx_array,
                                  const gpp_complex *wtilde_array, const gpp_complex *aqsmtemp,
                                  const gpp_complex *aqsntemp, const gpp_complex *I_eps_array,
                                  const double *vcoul, double occ) {
    gpp_problem q{};
    q.number_bands = number_bands;
    q.nvband = nvband;
    q.ncouls = ncouls;
    q.ngpown = ngpown;
    q.nw = 3;  // nstart = 0, nend = 3 (GPPComplex.cu:2-3)
    q.aqsmtemp = aqsmtemp;
    q.aqsntemp = aqsntemp;
    q.I_eps_array = I_eps_array;
    q.wtilde_array = wtilde_array;
    q.vcoul = vcoul;
    q.inv_igp_index = inv_igp_index;
    q.wx_array = wx_array;
    q.wx_stride = 0;
    q.occ = occ;
    q.semantics = GPP_SEM_COMPLEX_SEQ;
    q.precision = dropin_precision();
    return q;
}

gpp_status gpp_till_nvband(int nvband, int ngpown, int ncouls, const int *inv_igp_index,
                           const double *wx_array, const gpp_complex *wtilde_array,
                           const gpp_complex *aqsmtemp, const gpp_complex *aqsntemp,
                           const gpp_complex *I_eps_array, gpp_complex *asxtemp, const double *vcoul,
                           gpp_complex *acht_n1_loc, double *achtemp_re, double *achtemp_im,
                           double occ) {
    gpp_problem q = compat_problem(nvband, nvband, ngpown, ncouls, inv_igp_index, wx_array,
                                   wtilde_array, aqsmtemp, aqsntemp, I_eps_array, vcoul, occ);
    gpp_status st = validate(&q);
    if (st != GPP_OK) return st;
    if (!achtemp_re || !achtemp_im || !asxtemp)
        return fail(GPP_ERR_INVALID_ARGUMENT, "achtemp_re/achtemp_im/asxtemp is NULL");
    OutSpec o;
    o.ach_re = achtemp_re;
    o.ach_im = achtemp_im;
    o.asx = reinterpret_cast<double2 *>(asxtemp);
    o.n1 = reinterpret_cast<double2 *>(acht_n1_loc);
    o.accumulate = 1;
    return run_sigma(to_problem(q), 0, nvband, q.precision, o, true, t_compat_stream);
}

gpp_status gpp_noflag_occ_solver(int number_bands, int nvband, int ngpown, int ncouls,
                                 const int *inv_igp_index, const double *wx_array,
                                 const gpp_complex *wtilde_array, const gpp_complex *aqsmtemp,
                                 const gpp_complex *aqsntemp, const gpp_complex *I_eps_array,
                                 const double *vcoul, double *achtemp_re, double *achtemp_im,
                                 gpp_complex *acht_n1_loc) {
    gpp_problem q = compat_problem(number_bands, nvband, ngpown, ncouls, inv_igp_index, wx_array,
                                   wtilde_array, aqsmtemp, aqsntemp, I_eps_array, vcoul, 1.0);
    gpp_status st = validate(&q);
    if (st != GPP_OK) return st;
    if (!achtemp_re || !achtemp_im) return fail(GPP_ERR_INVALID_ARGUMENT, "achtemp_re/im is NULL");
    OutSpec o;
    o.ach_re = achtemp_re;
    o.ach_im = achtemp_im;
    o.n1 = reinterpret_cast<double2 *>(acht_n1_loc);
    o.accumulate = 1;
    return run_sigma(to_problem(q), nvband, number_bands, q.precision, o, true, t_compat_stream);
}

static gpp_status reduce_achstemp_impl(int number_bands, const int *inv_igp_index, int ncouls,
                                       const gpp_complex *aqsmtemp, const gpp_complex *aqsntemp,
                                       const gpp_complex *I_eps_array, int ngpown,
                                       const double *vcoul, OutSpec o) {
    static const double dummy_wx = 0.0;  // the static term has no frequency
    gpp_problem q = compat_problem(number_bands, 0, ngpown, ncouls, inv_igp_index, &dummy_wx,
                                   I_eps_array, aqsmtemp, aqsntemp, I_eps_array, vcoul, 1.0);
    gpp_status st = validate(&q);
    if (st != GPP_OK) return st;
    o.accumulate = 1;
    return run_sigma(to_problem(q), 0, number_bands, GPP_PRECISION_FP64, o, false, t_compat_stream);
}

gpp_status gpp_reduce_achstemp(int number_bands, const int *inv_igp_index, int ncouls,
                               const gpp_complex *aqsmtemp, const gpp_complex *aqsntemp,
                               const gpp_complex *I_eps_array, gpp_complex *achstemp, int ngpown,
                               const double *vcoul) {
    if (!achstemp) return fail(GPP_ERR_INVALID_ARGUMENT, "achstemp is NULL");
    OutSpec o;
    o.achs = reinterpret_cast<double2 *>(achstemp);
    return reduce_achstemp_impl(number_bands, inv_igp_index, ncouls, aqsmtemp, aqsntemp,
                                I_eps_array, ngpown, vcoul, o);
}

// Split real/imaginary destination, for the reference's d_reduce_achstemp
// signature (GPPComplex.h:308); used by gpp_compat.cpp.
gpp_status gpp_reduce_achstemp_split(int number_bands, const int *inv_igp_index, int ncouls,
                                     const gpp_complex *aqsmtemp, const gpp_complex *aqsntemp,
                                     const gpp_complex *I_eps_array, double *re, double *im,
                                     int ngpown, const double *vcoul) {
    if (!re || !im) return fail(GPP_ERR_INVALID_ARGUMENT, "achstemp_re/im is NULL");
    OutSpec o;
    o.achs_re = re;
    o.achs_im = im;
    return reduce_achstemp_impl(number_bands, inv_igp_index, ncouls, aqsmtemp, aqsntemp,
                                I_eps_array, ngpown, vcoul, o);
}

gpp_status gpp_wait(gpp_stream_t stream, int timeout_ms) {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t q = cudaStreamQuery(s);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) return cuda_fail(q, "cudaStreamQuery");
        if (timeout_ms >= 0) {
            auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
                          std::chrono::steady_clock::now() - t0).count();
            if (ms >= timeout_ms) return fail(GPP_ERR_NOT_READY, "stream still busy after %d ms", timeout_ms);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    int dev = 0;
    int *err = nullptr;
    gpp_status st = device_setup(&dev, &err);
    if (st != GPP_OK) return st;
    int h = 0;
    GPP_CUDA_TRY(cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost), "read fault word");
    if (h) {
        GPP_CUDA_TRY(cudaMemset(err, 0, sizeof(int)), "clear fault word");
        if (h & kErrPipelineTimeout)
            return fail(GPP_ERR_DEVICE_TIMEOUT,
                        "a kernel's shared-memory pipeline wait gave up; results are invalid");
        return fail(GPP_ERR_BAD_INDEX, "device saw %s%s",
                    (h & kErrBadIgp) ? "inv_igp_index < 0 " : "",
                    (h & kErrBadIndinv) ? "indinv out of [0, ncouls)" : "");
    }
    return GPP_OK;
}

// ---------------------------------------------------------------------------
// Host-buffer path: a context owns device copies of the inputs and outputs.
// Input copies run on their own stream in pieces -- the band arrays first,
// then the G' rows in row-pair ranges -- and the kernels of each piece start
// as soon as its rows have landed, so the copies overlap the computation.
struct gpp_context {
    cudaStream_t stream = nullptr;  // kernels and the result copy
    cudaStream_t copy = nullptr;    // input copies
    void *dev = nullptr;
    size_t dev_bytes = 0;
    int device = 0;
    // Copy start, copy end, compute start, compute end, result copy end.
    cudaEvent_t ev[5] = {};
    cudaEvent_t bands_ready = nullptr, done = nullptr;
    cudaEvent_t ready[kMaxRowPieces] = {};
    // Timing twins of the copy milestones (bands landed, piece k landed) and
    // the compute stream's start of each piece, for gpp_context_last_trace.
    cudaEvent_t t_bands = nullptr;
    cudaEvent_t t_ready[kMaxRowPieces] = {}, t_started[kMaxRowPieces] = {};
    int pieces = 0;
    bool timed = false;
};

// Row pieces of the host path, in sixteenths of the row pairs: a small first
// piece so the kernels start early, then larger ones.  Each piece is copied
// while the previous ones compute (the link moves rows ~25x faster than the
// kernels consume them), and fewer pieces mean fewer partial last waves of
// the unoccupied-band kernel.
constexpr int kHostPieceCuts[] = {1, 5, 16};

// How gpp_sigma_host moves inputs the device can address (pinned host
// memory): 1 = an SM pull kernel (default), 0 = the copy engine
// (GPP_HOST_PULL=ce).  Measured on GB300 at the production shape from
// pinned memory, copy-engine copies ran either at ~210 GB/s or at 10-40 GB/s,
// alternating between back-to-back calls and always slow after the GPU had
// been idle for a fraction of a second (calls of 218 or 263-287 ms); the
// pull kernel moved the same 2.25 GB in 10.7-11 ms on every call, and the
// call took 224 ms back to back and after idle pauses alike.  Pageable
// memory always goes through the copy engine.
int host_pull_mode() {
    static const int mode = [] {
        const char *v = getenv("GPP_HOST_PULL");
        return (v && strcmp(v, "ce") == 0) ? 0 : 1;
    }();
    return mode;
}

// The piece cuts in effect: GPP_HOST_PIECES="c1,c2,...,16" (increasing
// sixteenths ending at 16, at most kMaxRowPieces of them) overrides the
// default, for hosts whose links move rows at another speed.
std::vector<int> host_piece_cuts() {
    static const std::vector<int> cuts = [] {
        std::vector<int> v;
        if (const char *env = getenv("GPP_HOST_PIECES")) {
            int last = 0;
            for (const char *c = env; *c;) {
                char *end = nullptr;
                const long x = strtol(c, &end, 10);
                if (end == c || x <= last || x > 16) { v.clear(); break; }
                v.push_back((int)x);
                last = (int)x;
                c = (*end == ',') ? end + 1 : end;
                if (*end && *end != ',') { v.clear(); break; }
            }
            if (v.empty() || v.back() != 16 || (int)v.size() > kMaxRowPieces) v.clear();
        }
        if (v.empty()) v.assign(std::begin(kHostPieceCuts), std::end(kHostPieceCuts));
        return v;
    }();
    return cuts;
}

static void context_release(gpp_context *c) {
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->ready)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->t_ready)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->t_started)
        if (e) cudaEventDestroy(e);
    if (c->t_bands) cudaEventDestroy(c->t_bands);
    if (c->bands_ready) cudaEventDestroy(c->bands_ready);
    if (c->done) cudaEventDestroy(c->done);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

gpp_status gpp_context_create(gpp_context **ctx) {
    if (!ctx) return fail(GPP_ERR_INVALID_ARGUMENT, "ctx is NULL");
    gpp_context *c = new gpp_context();
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    // The copy stream at the highest priority: a pull kernel (GPP_HOST_PULL=sm)
    // on it is scheduled ahead of the computation's blocks.
    int prio_lo = 0, prio_hi = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithPriority(&c->copy, cudaStreamNonBlocking, prio_hi);
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
    for (int i = 0; i < kMaxRowPieces && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&c->ready[i], cudaEventDisableTiming);
    for (int i = 0; i < kMaxRowPieces && e == cudaSuccess; ++i) e = cudaEventCreate(&c->t_ready[i]);
    for (int i = 0; i < kMaxRowPieces && e == cudaSuccess; ++i) e = cudaEventCreate(&c->t_started[i]);
    if (e == cudaSuccess) e = cudaEventCreate(&c->t_bands);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->bands_ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        context_release(c);
        return cuda_fail(e, "gpp_context_create");
    }
    *ctx = c;
    return GPP_OK;
}

gpp_status gpp_context_destroy(gpp_context *ctx) {
    if (!ctx) return GPP_OK;
    if (ctx->copy) cudaStreamSynchronize(ctx->copy);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->dev) cudaFree(ctx->dev);
    context_release(ctx);
    return GPP_OK;
}

gpp_status gpp_sigma_host(gpp_context *ctx, const gpp_problem *problem, const gpp_outputs *out) {
    if (!ctx) return fail(GPP_ERR_INVALID_ARGUMENT, "ctx is NULL");
    gpp_status st = validate(problem);
    if (st != GPP_OK) return st;
    if (!out || !out->achtemp || !out->asxtemp)
        return fail(GPP_ERR_INVALID_ARGUMENT, "outputs achtemp/asxtemp are required");
    const gpp_problem &h = *problem;
    const size_t nb = (size_t)h.number_bands, nc = (size_t)h.ncouls, ng = (size_t)h.ngpown,
                 nw = (size_t)h.nw;
    const size_t wx_n = h.wx_stride ? nb * (size_t)h.wx_stride : nw;
    struct Seg { const void *src; size_t bytes; size_t off; };
    enum { kAqsm, kAqsn, kIeps, kWt, kVcoul, kInvIgp, kIndinv, kWx };
    std::vector<Seg> in = {
        {h.aqsmtemp, nb * nc * 16, 0}, {h.aqsntemp, nb * nc * 16, 0},
        {h.I_eps_array, ng * nc * 16, 0}, {h.wtilde_array, ng * nc * 16, 0},
        {h.vcoul, nc * 8, 0}, {h.inv_igp_index, ng * 4, 0},
        {h.indinv, h.indinv ? nc * 4 : 0, 0}, {h.wx_array, wx_n * 8, 0}};
    size_t off = 0;
    for (auto &sg : in) { sg.off = off; off = align_up(off + sg.bytes); }
    const size_t o_out = off;
    off = align_up(off + 16 * (2 * nw + (out->acht_n1_loc ? nb : 0) + 1));
    if (off > ctx->dev_bytes) {
        if (ctx->dev) {
            cudaStreamSynchronize(ctx->copy);
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->dev);
            ctx->dev = nullptr;
            ctx->dev_bytes = 0;
        }
        GPP_CUDA_TRY(cudaMalloc(&ctx->dev, off), "cudaMalloc(context buffers)");
        ctx->dev_bytes = off;
    }
    char *d = static_cast<char *>(ctx->dev);
    ctx->timed = false;
    // Transfers: the SMs pull every input the device can address (pinned
    // host memory, 16-byte aligned) with a kernel on the copy stream (highest
    // priority, so its blocks take SM slots as the computation's blocks
    // retire); anything else, or everything with GPP_HOST_PULL=ce, goes
    // through the copy engine.
    const bool sm_pull = host_pull_mode() == 1;
    std::vector<const char *> src_dev(in.size(), nullptr);
    if (sm_pull)
        for (size_t k = 0; k < in.size(); ++k) {
            void *dp = nullptr;
            if (in[k].bytes && ((uintptr_t)in[k].src & 15) == 0 && (in[k].bytes & 15) == 0 &&
                cudaHostGetDevicePointer(&dp, const_cast<void *>(in[k].src), 0) == cudaSuccess)
                src_dev[k] = static_cast<const char *>(dp);
            else
                cudaGetLastError();  // not device-accessible: the copy engine moves it
        }
    auto h2d = [&](int k, size_t from, size_t bytes) {
        if (src_dev[k] && (from & 15) == 0 && (bytes & 15) == 0)
            return launch_host_pull(d + in[k].off + from, src_dev[k] + from, bytes, ctx->copy);
        return cudaMemcpyAsync(d + in[k].off + from, static_cast<const char *>(in[k].src) + from,
                               bytes, cudaMemcpyHostToDevice, ctx->copy);
    };
    // Copies may only overwrite the buffers once the previous call is done.
    GPP_CUDA_TRY(cudaStreamWaitEvent(ctx->copy, ctx->done, 0), "cudaStreamWaitEvent");
    GPP_CUDA_TRY(cudaEventRecord(ctx->ev[0], ctx->copy), "cudaEventRecord");
    for (int k : {kVcoul, kInvIgp, kIndinv, kWx, kAqsm, kAqsn})
        if (in[k].bytes) GPP_CUDA_TRY(h2d(k, 0, in[k].bytes), "cudaMemcpyAsync(H2D)");
    GPP_CUDA_TRY(cudaEventRecord(ctx->bands_ready, ctx->copy), "cudaEventRecord");
    GPP_CUDA_TRY(cudaEventRecord(ctx->t_bands, ctx->copy), "cudaEventRecord");
    RowPieces pieces;
    const int pairs = (int)((ng + 1) / 2);
    pieces.n = 0;
    pieces.pair[0] = 0;
    for (int cut : host_piece_cuts()) {
        const int b = (int)((long long)pairs * cut / 16);
        if (b > pieces.pair[pieces.n]) pieces.pair[++pieces.n] = b;
    }
    if (pieces.n == 0) pieces.pair[++pieces.n] = 0;  // no rows: one empty piece
    for (int k = 0; k < pieces.n; ++k) {
        const size_t r0 = 2 * (size_t)pieces.pair[k];
        const size_t r1 = std::min(2 * (size_t)pieces.pair[k + 1], ng);
        if (r1 > r0) {
            GPP_CUDA_TRY(h2d(kWt, r0 * nc * 16, (r1 - r0) * nc * 16), "cudaMemcpyAsync(H2D)");
            GPP_CUDA_TRY(h2d(kIeps, r0 * nc * 16, (r1 - r0) * nc * 16), "cudaMemcpyAsync(H2D)");
        }
        pieces.ready[k] = ctx->ready[k];
        pieces.started[k] = ctx->t_started[k];
        GPP_CUDA_TRY(cudaEventRecord(ctx->ready[k], ctx->copy), "cudaEventRecord");
        GPP_CUDA_TRY(cudaEventRecord(ctx->t_ready[k], ctx->copy), "cudaEventRecord");
    }
    ctx->pieces = pieces.n;
    GPP_CUDA_TRY(cudaEventRecord(ctx->ev[1], ctx->copy), "cudaEventRecord");

    gpp_problem q = h;
    q.aqsmtemp = reinterpret_cast<const gpp_complex *>(d + in[kAqsm].off);
    q.aqsntemp = reinterpret_cast<const gpp_complex *>(d + in[kAqsn].off);
    q.I_eps_array = reinterpret_cast<const gpp_complex *>(d + in[kIeps].off);
    q.wtilde_array = reinterpret_cast<const gpp_complex *>(d + in[kWt].off);
    q.vcoul = reinterpret_cast<const double *>(d + in[kVcoul].off);
    q.inv_igp_index = reinterpret_cast<const int *>(d + in[kInvIgp].off);
    q.indinv = h.indinv ? reinterpret_cast<const int *>(d + in[kIndinv].off) : nullptr;
    q.wx_array = reinterpret_cast<const double *>(d + in[kWx].off);
    gpp_complex *dout = reinterpret_cast<gpp_complex *>(d + o_out);
    gpp_outputs o{};
    o.achtemp = dout;
    o.asxtemp = dout + nw;
    o.achstemp = dout + 2 * nw;
    o.acht_n1_loc = out->acht_n1_loc ? dout + 2 * nw + 1 : nullptr;
    if (!out->achstemp) o.achstemp = nullptr;
    GPP_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->bands_ready, 0), "cudaStreamWaitEvent");
    GPP_CUDA_TRY(cudaEventRecord(ctx->ev[2], ctx->stream), "cudaEventRecord");
    st = sigma_impl(&q, &o, ctx->stream, &pieces);
    if (st == GPP_OK) {
        // The kernels waited on every piece; make the ordering explicit for
        // the zero-row case too.
        cudaError_t e = cudaStreamWaitEvent(ctx->stream, ctx->ev[1], 0);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaStreamWaitEvent");
    }
    cudaEventRecord(ctx->done, ctx->stream);
    if (st != GPP_OK) return st;
    GPP_CUDA_TRY(cudaEventRecord(ctx->ev[3], ctx->stream), "cudaEventRecord");
    const size_t out_bytes = 16 * (2 * nw + 1 + (out->acht_n1_loc ? nb : 0));
    std::vector<gpp_complex> tmp(out_bytes / 16);
    GPP_CUDA_TRY(cudaMemcpyAsync(tmp.data(), dout, out_bytes, cudaMemcpyDeviceToHost, ctx->stream),
                 "cudaMemcpyAsync(D2H)");
    GPP_CUDA_TRY(cudaEventRecord(ctx->ev[4], ctx->stream), "cudaEventRecord");
    GPP_CUDA_TRY(cudaEventRecord(ctx->done, ctx->stream), "cudaEventRecord");
    st = gpp_wait(reinterpret_cast<gpp_stream_t>(ctx->stream), -1);
    if (st != GPP_OK) return st;
    ctx->timed = true;
    memcpy(out->achtemp, tmp.data(), 16 * nw);
    memcpy(out->asxtemp, tmp.data() + nw, 16 * nw);
    if (out->achstemp) out->achstemp[0] = tmp[2 * nw];
    if (out->acht_n1_loc) memcpy(out->acht_n1_loc, tmp.data() + 2 * nw + 1, 16 * nb);
    return GPP_OK;
}

gpp_status gpp_context_last_timing(gpp_context *ctx, float *h2d_ms, float *compute_ms,
                                   float *d2h_ms) {
    if (!ctx) return fail(GPP_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!ctx->timed) return fail(GPP_ERR_NOT_READY, "no completed gpp_sigma_host call");
    if (h2d_ms) GPP_CUDA_TRY(cudaEventElapsedTime(h2d_ms, ctx->ev[0], ctx->ev[1]), "cudaEventElapsedTime");
    if (compute_ms)
        GPP_CUDA_TRY(cudaEventElapsedTime(compute_ms, ctx->ev[2], ctx->ev[3]), "cudaEventElapsedTime");
    if (d2h_ms) GPP_CUDA_TRY(cudaEventElapsedTime(d2h_ms, ctx->ev[3], ctx->ev[4]), "cudaEventElapsedTime");
    return GPP_OK;
}

gpp_status gpp_context_last_trace(gpp_context *ctx, float *ms, int capacity, int *count) {
    if (!ctx || !count) return fail(GPP_ERR_INVALID_ARGUMENT, "ctx/count is NULL");
    if (!ctx->timed) return fail(GPP_ERR_NOT_READY, "no completed gpp_sigma_host call");
    const int n = 1 + 2 * ctx->pieces;
    *count = n;
    if (!ms || capacity < n) return fail(GPP_ERR_INVALID_ARGUMENT, "trace needs %d floats", n);
    GPP_CUDA_TRY(cudaEventElapsedTime(&ms[0], ctx->ev[0], ctx->t_bands), "cudaEventElapsedTime");
    for (int k = 0; k < ctx->pieces; ++k) {
        GPP_CUDA_TRY(cudaEventElapsedTime(&ms[1 + 2 * k], ctx->ev[0], ctx->t_ready[k]),
                     "cudaEventElapsedTime");
        GPP_CUDA_TRY(cudaEventElapsedTime(&ms[2 + 2 * k], ctx->ev[0], ctx->t_started[k]),
                     "cudaEventElapsedTime");
    }
    return GPP_OK;
}

int gpp_variant_count(void) { return mixed_variant_count(); }
const char *gpp_variant_name(int variant) { return mixed_variant_name(variant); }

gpp_status gpp_set_variant(int nw, int variant) {
    if (nw <= 0 || variant < -1 || variant >= mixed_variant_count())
        return fail(GPP_ERR_INVALID_ARGUMENT, "bad nw or variant");
    if (variant >= 0 && !mixed_variant_valid(variant, nw))
        return fail(GPP_ERR_UNSUPPORTED, "variant %d is not compiled for %d frequencies", variant, nw);
    int dev = 0;
    GPP_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    tune_cache_load_locked();
    g_tuned[dev & 255][nwc_of(nw)] = variant + 1;  // -1 clears back to the default
    return GPP_OK;
}

gpp_status gpp_tuned_variant(int nw, int *variant) {
    if (nw <= 0 || !variant) return fail(GPP_ERR_INVALID_ARGUMENT, "bad nw or NULL output");
    int dev = 0;
    GPP_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    *variant = mixed_variant_for(dev, nw);
    return GPP_OK;
}

gpp_status gpp_autotune(const gpp_problem *problem, int max_bands, gpp_stream_t stream,
                        int *best) {
    gpp_status st = validate(problem);
    if (st != GPP_OK) return st;
    if (problem->precision != GPP_PRECISION_MIXED)
        return fail(GPP_ERR_UNSUPPORTED, "the autotuner selects mixed-precision variants");
    Problem p = to_problem(*problem);
    // Time the unoccupied bands only (the variants differ there), at most
    // max_bands of them.
    const int unocc = p.nb - p.nv;
    if (unocc <= 0 || p.ng == 0) return fail(GPP_ERR_INVALID_ARGUMENT, "no unoccupied bands to time");
    const int nbt = (max_bands > 0 && max_bands < unocc) ? max_bands : unocc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0;
    GPP_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    double2 *out = nullptr;
    st = workspace_alloc(reinterpret_cast<void **>(&out), sizeof(double2) * 2 * (size_t)p.nw, s);
    if (st != GPP_OK) return st;
    OutSpec o;
    o.ach = out;
    o.asx = out + p.nw;
    cudaEvent_t e0, e1;
    GPP_CUDA_TRY(cudaEventCreate(&e0), "cudaEventCreate");
    GPP_CUDA_TRY(cudaEventCreate(&e1), "cudaEventCreate");
    float best_ms = 0.f;
    int best_v = -1;
    const bool timing = t_timing;
    t_timing = false;
    for (int v = 0; v < mixed_variant_count() && st == GPP_OK; ++v) {
        if (!mixed_variant_valid(v, p.nw)) continue;
        t_force_variant = v;
        float vbest = 0.f;
        for (int rep = 0; rep < 3 && st == GPP_OK; ++rep) {
            cudaEventRecord(e0, s);
            st = run_sigma(p, p.nv, p.nv + nbt, GPP_PRECISION_MIXED, o, true, s);
            cudaEventRecord(e1, s);
            if (st != GPP_OK) break;
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) { st = cuda_fail(e, "autotune"); break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && (vbest == 0.f || ms < vbest)) vbest = ms;  // rep 0 warms up
        }
        if (st == GPP_OK && (best_v < 0 || vbest < best_ms)) {
            best_ms = vbest;
            best_v = v;
        }
    }
    t_force_variant = -1;
    t_timing = timing;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    if (st != GPP_OK) return st;
    {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        tune_cache_load_locked();
        g_tuned[dev & 255][nwc_of(p.nw)] = best_v + 1;
        tune_cache_save_locked();
    }
    if (best) *best = best_v;
    return GPP_OK;
}

gpp_status gpp_enable_kernel_timing(int enable) {
    t_timing = enable != 0;
    if (t_timing && !t_ev0) {
        GPP_CUDA_TRY(cudaEventCreate(&t_ev0), "cudaEventCreate");
        GPP_CUDA_TRY(cudaEventCreate(&t_ev1), "cudaEventCreate");
    }
    t_timed = false;
    return GPP_OK;
}

gpp_status gpp_last_kernel_ms(float *ms) {
    if (!ms) return fail(GPP_ERR_INVALID_ARGUMENT, "ms is NULL");
    if (!t_timed) return fail(GPP_ERR_NOT_READY, "no timed kernel yet (enable timing first)");
    GPP_CUDA_TRY(cudaEventSynchronize(t_ev1), "cudaEventSynchronize");
    GPP_CUDA_TRY(cudaEventElapsedTime(ms, t_ev0, t_ev1), "cudaEventElapsedTime");
    return GPP_OK;
}

gpp_status gpp_selftest_wait_timeout(int polls, gpp_stream_t stream) {
    if (polls < 1 || polls > kWaitLimit) return fail(GPP_ERR_INVALID_ARGUMENT, "polls out of range");
    int dev = 0;
    int *err = nullptr;
    gpp_status st = device_setup(&dev, &err);
    if (st != GPP_OK) return st;
    cudaError_t e = launch_wait_selftest(err, polls, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "wait self-test launch");
    return GPP_OK;
}

gpp_status gpp_probe_fma_peaks(double *fp64_tflops, double *fp32_tflops) {
    if (!fp64_tflops || !fp32_tflops) return fail(GPP_ERR_INVALID_ARGUMENT, "NULL output");
    cudaError_t e = probe_fma_peaks(fp64_tflops, fp32_tflops);
    if (e != cudaSuccess) return cuda_fail(e, "FMA probe");
    return GPP_OK;
}

}  // extern "C"

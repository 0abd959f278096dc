// gpp_batched.cu -- many quasiparticle states in one persistent launch.
//
// A batch plan lists every tile of every state -- occupied-band tiles (one
// band x RG rows) and unoccupied-band tiles (RN bands x RG rows), for each
// frequency chunk -- as work items in two lists, each ordered longest first.
// Each list runs as its own persistent launch (resident blocks x SMs) whose
// blocks pop items from a global counter: the occupied-band tile keeps its
// branchy body and register count out of the unoccupied-band kernel.  Each
// item writes its partial sums to a fixed slot, so the result does not
// depend on which block ran which item, and one batched fixed-order
// reduction produces every state's outputs.
//
// Mixed precision needs each state's float-float split planes; states are
// grouped into waves whose planes fit a workspace budget, and each wave runs
// its prep kernels then one persistent launch.  The whole sequence is
// enqueued on one stream and, on a capturable stream, recorded once into a
// CUDA graph that later runs replay.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gpp_gb300.h"
#include "gpp_kernels.h"
#include "gpp_tiles_fp64.cuh"
#include "gpp_tiles_mixed.cuh"

namespace gpp {

gpp_status set_error(gpp_status s, const char *msg);

namespace {

constexpr int kThreads = 128;  // every tile family runs 4 warps

// Reduction job: dst[k] (=|+=) sum_t src[k*stride + t], k < nseg, t < len.
struct ReduceJob {
    const double2 *src;
    long long stride;
    int len, nseg;
    double2 *dst;
    int accumulate;
};

template <int THREADS>
__global__ void __launch_bounds__(THREADS)
batched_reduce_kernel(const ReduceJob *jobs, const int *seg_prefix, int njobs) {
    __shared__ double red[(THREADS / 32) * 2];
    __shared__ double S[2];
    // Find the job of this block's segment (prefix sums of nseg).
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (seg_prefix[mid] <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const ReduceJob j = jobs[lo];
    const int k = blockIdx.x - seg_prefix[lo];
    const double2 *seg = j.src + (long long)k * j.stride;
    double v[2] = {0.0, 0.0};
    for (int t = threadIdx.x; t < j.len; t += THREADS) {
        const double2 x = seg[t];
        v[0] += x.x;
        v[1] += x.y;
    }
    block_reduce<2, THREADS>(v, red, S);
    if (threadIdx.x == 0) {
        double2 r = make_double2(S[0], S[1]);
        if (j.accumulate) r = cadd(j.dst[k], r);
        j.dst[k] = r;
    }
}

// Persistent FP64 kernel over a list of tiles.
template <int RN, int RG, int NWC>
__global__ void __launch_bounds__(kThreads)
batched_fp64_kernel(const Problem *probs, const Partials *parts, const BatchItem *items,
                    int n_items, int *head) {
    constexpr int KN = RN * RG * NWC * 2, KF = RG * NWC * 4;
    constexpr int K = KN > KF ? KN : KF;
    __shared__ double red[(kThreads / 32) * K];
    __shared__ double S[K];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) return;
        const BatchItem bi = items[it];
        const Problem p = probs[bi.state];
        const Partials part = parts[bi.state];
        if (bi.kind == 0) {
            if (p.semantics == kSemKerSeq)
                flag_fp64_tile<RG, NWC, kThreads, kSemKerSeq>(p, part, bi.row_tile, bi.band_tile,
                                                              bi.iw_chunk, bi.tile, red, S);
            else
                flag_fp64_tile<RG, NWC, kThreads, kSemComplexSeq>(
                    p, part, bi.row_tile, bi.band_tile, bi.iw_chunk, bi.tile, red, S);
        } else {
            noflag_fp64_tile<RN, RG, NWC, kThreads>(p, part, p.nv, p.nb, bi.row_tile,
                                                    bi.band_tile, bi.iw_chunk, bi.tile, red, S);
        }
        __syncthreads();
    }
}

// Persistent mixed-precision kernels: occupied-band tiles (float-float,
// register-heavy) and unoccupied-band tiles (shared-memory pipeline) run as
// two launches so each keeps its own occupancy.
template <int NWC, int FRG>
__global__ void __launch_bounds__(kThreads, NWC <= 4 ? 3 : 2)
batched_flag_mixed_kernel(const Problem *probs, const Partials *parts, const SplitPlanes *splits,
                          const BatchItem *items, int n_items, int *head) {
    constexpr int KF = FRG * NWC * 4;
    __shared__ double red[(kThreads / 32) * KF];
    __shared__ double S[KF];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) return;
        const BatchItem bi = items[it];
        const Problem p = probs[bi.state];
        const Partials part = parts[bi.state];
        const SplitPlanes sp = splits[bi.state];
        if (p.semantics == kSemKerSeq)
            flag_mixed_tile<FRG, NWC, kThreads, kSemKerSeq>(p, part, sp, bi.row_tile, bi.band_tile,
                                                            bi.iw_chunk, bi.tile, red, S);
        else
            flag_mixed_tile<FRG, NWC, kThreads, kSemComplexSeq>(
                p, part, sp, bi.row_tile, bi.band_tile, bi.iw_chunk, bi.tile, red, S);
        __syncthreads();
    }
}

// Columns per pipeline chunk of the persistent mixed kernel: the fastest
// block-sync chunk of the single-state kernel measured on GB300 (192 columns
// for up to 4 frequencies, 256 for the 8-frequency tile).
template <int NWC>
__host__ __device__ constexpr int batch_kc() { return NWC <= 4 ? 192 : 256; }

// Resident blocks as the single-state kernel: 4 (128 registers) up to 4
// frequencies, 3 (168 registers) for the 8-frequency tile.  Left to the
// compiler's heuristic, the persistent loop takes 158 and 254 registers and
// a quarter to a third of the warps.
// NWARP warps per block, one band each: 4 (the default tile, 4 bands x 2
// rows) or 8 (8 bands x 2 rows), following the tile shape the autotuner
// chose for single states; the same register budget per thread either way.
template <int RG, int NWC, int NWARP = 4>
__global__ void __launch_bounds__(NWARP * 32, (NWC <= 4 ? 4 : 3) * 4 / NWARP)
batched_noflag_mixed_kernel(const Problem *probs, const Partials *parts, const SplitPlanes *splits,
                            const BatchItem *items, int n_items, int *head) {
    __shared__ int s_item;
    bool reinit = false;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) return;
        const BatchItem bi = items[it];
        const Problem p = probs[bi.state];
        const Partials part = parts[bi.state];
        const SplitPlanes sp = splits[bi.state];
        if (!mixed_tile<1, RG, NWC, NWARP, batch_kc<NWC>(), 2, kSyncBlock>(
                p, part, sp, p.nv, p.nb, bi.row_tile, bi.band_tile, bi.iw_chunk, bi.tile, reinit))
            return;  // abandoned after a bounded wait; the fault bit is set
        reinit = true;
        __syncthreads();
    }
}

template <typename K>
int resident_blocks(K kern, size_t smem, int threads = kThreads) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem);
    return std::max(1, sms) * std::max(1, per);
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace gpp

using namespace gpp;

// A batch of states prepared once and run many times.
struct gpp_batch {
    int device = 0, nstates = 0, precision = 0, nw = 0;
    std::vector<Problem> probs;
    std::vector<Partials> parts;
    std::vector<SplitPlanes> splits;
    std::vector<BatchItem> items;
    struct Wave {
        int s0, s1;      // states [s0, s1)
        int i0, i_mid, i1;  // occupied items [i0, i_mid), unoccupied [i_mid, i1)
        size_t split_bytes;
        std::vector<size_t> split_off;  // per state in the wave
    };
    std::vector<Wave> waves;
    std::vector<ReduceJob> jobs;
    std::vector<int> seg_prefix;
    int total_segs = 0;
    // Static term: per state, [partials] and a destination.
    std::vector<std::pair<int, double2 *>> achs;  // (state, dst) for states that want it
    char *dev = nullptr;  // one allocation: tables, partials, counters, split workspace
    size_t dev_bytes = 0;
    Problem *d_probs = nullptr;
    Partials *d_parts = nullptr;
    SplitPlanes *d_splits = nullptr;
    BatchItem *d_items = nullptr;
    ReduceJob *d_jobs = nullptr;
    int *d_prefix = nullptr;
    int *d_heads = nullptr;
    char *d_split = nullptr;
    std::vector<int> achs_blocks;
    std::vector<std::pair<double2 *, size_t>> n1_zero;
    int launches_per_run = 0;
    int warps = 4;    // warps (bands) per unoccupied-band block of the mixed path
    size_t smem = 0;  // persistent kernel: dynamic shared memory per block
    int grid = 1;       // persistent kernels: resident blocks on the device
    int grid_flag = 1;
    cudaGraphExec_t graph = nullptr;
    int *err = nullptr;
};

namespace {

gpp_status plan_batch(gpp_batch *b, const gpp_problem *problems, const gpp_outputs *outs,
                      int nstates, size_t split_budget) {
    const int precision = problems[0].precision;
    const int nw = problems[0].nw;
    const int sem = problems[0].semantics;
    for (int i = 0; i < nstates; ++i) {
        const gpp_problem &q = problems[i];
        if (q.precision != precision || q.nw != nw || q.semantics != sem)
            return set_error(GPP_ERR_UNSUPPORTED,
                             "a batch needs one precision, one nw and one semantics");
        if (!outs[i].achtemp || !outs[i].asxtemp)
            return set_error(GPP_ERR_INVALID_ARGUMENT, "outputs achtemp/asxtemp are required");
        if (outs[i].acht_n1_loc && nw < 3)
            return set_error(GPP_ERR_INVALID_ARGUMENT, "acht_n1_loc needs nw >= 3");
        if (q.number_bands < 0 || q.nvband < 0 || q.nvband > q.number_bands || q.ncouls <= 0 ||
            q.ngpown < 0 || nw <= 0 || (q.wx_stride != 0 && q.wx_stride < nw) ||
            (q.number_bands > 0 && (!q.aqsmtemp || !q.aqsntemp)) ||
            (q.ngpown > 0 && (!q.I_eps_array || !q.wtilde_array || !q.inv_igp_index)) ||
            !q.vcoul || !q.wx_array)
            return set_error(GPP_ERR_INVALID_ARGUMENT, "invalid problem in batch");
    }
    b->nstates = nstates;
    b->precision = precision;
    b->nw = nw;
    const bool mixed = precision == GPP_PRECISION_MIXED;
    const int nwc = nw <= 4 ? nw : 8;
    const int nchunk = (nw + nwc - 1) / nwc;

    // Tile geometry shared by the planner and the kernels.
    Problem p0{};
    p0.nw = nw;
    const TileShape fs = flag_shape(p0);
    // The unoccupied-band tile shape of the mixed path follows the tuned
    // variant where the persistent kernel is compiled in that shape (4 or 8
    // warps of one band; 8 for 3- and 8-frequency chunks); otherwise, and for
    // a two-bands-per-warp choice, 4 bands x 2 rows.
    TileShape ns = fp64_noflag_shape(p0);
    if (mixed) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
        ns = mixed_noflag_shape(p0, tuned_mixed_variant(dev, nw));
        const bool eight = ns.threads == 256 && ns.rn == 8 && (nwc == 3 || nwc == 8);
        if (!eight) ns = mixed_noflag_shape(p0, mixed_default_variant());
        b->warps = eight ? 8 : 4;
    }

    struct StateGeom {
        long long rows_f, rows_n, tiles_f, tiles_n, ach_seg, n1_seg;
        size_t off_ach, off_asx, off_n1, off_achs;
        size_t split;
        int achs_blocks;
    };
    std::vector<StateGeom> g(nstates);
    size_t off = 0;
    auto reserve = [&](size_t bytes) { size_t o = off; off = align256(off + bytes); return o; };
    const size_t off_probs = reserve(sizeof(Problem) * nstates);
    const size_t off_parts = reserve(sizeof(Partials) * nstates);
    const size_t off_splits = reserve(sizeof(SplitPlanes) * nstates);
    for (int i = 0; i < nstates; ++i) {
        const gpp_problem &q = problems[i];
        Problem p{};
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
        p.nw = nw;
        p.occ = q.occ;
        p.semantics = q.semantics;
        b->probs.push_back(p);
        StateGeom &s = g[i];
        const bool hf = p.nv > 0 && p.ng > 0, hn = p.nb > p.nv && p.ng > 0;
        s.rows_f = hf ? ceil_div(p.ng, fs.rg) : 0;
        s.rows_n = hn ? ceil_div(p.ng, ns.rg) : 0;
        s.tiles_f = hf ? s.rows_f * p.nv : 0;
        s.tiles_n = hn ? s.rows_n * ceil_div(p.nb - p.nv, ns.rn) : 0;
        s.ach_seg = s.tiles_f + s.tiles_n;
        s.n1_seg = std::max(s.rows_f, s.rows_n);
        s.off_ach = reserve(sizeof(double2) * (size_t)(s.ach_seg * nw));
        s.off_asx = reserve(sizeof(double2) * (size_t)(s.tiles_f * nw));
        s.off_n1 = outs[i].acht_n1_loc && p.ng > 0 ? reserve(sizeof(double2) * (size_t)(s.n1_seg * p.nb)) : 0;
        s.achs_blocks = outs[i].achstemp && p.ng > 0 ? achstemp_blocks(p) : 0;
        s.off_achs = s.achs_blocks ? reserve(sizeof(double2) * s.achs_blocks) : 0;
        s.split = mixed ? align256(mixed_split_bytes(p)) : 0;
    }
    // Waves (mixed): consecutive states whose split planes fit the budget.
    std::vector<std::pair<int, int>> wave_states;
    size_t max_wave = 0;
    if (mixed) {
        int s0 = 0;
        size_t acc = 0;
        for (int i = 0; i < nstates; ++i) {
            if (i > s0 && acc + g[i].split > split_budget) {
                wave_states.push_back({s0, i});
                max_wave = std::max(max_wave, acc);
                s0 = i;
                acc = 0;
            }
            acc += g[i].split;
        }
        wave_states.push_back({s0, nstates});
        max_wave = std::max(max_wave, acc);
    } else {
        wave_states.push_back({0, nstates});
    }
    const size_t off_heads = reserve(sizeof(int) * 2 * wave_states.size());
    // Items per wave.
    for (auto &ws : wave_states) {
        gpp_batch::Wave w;
        w.s0 = ws.first;
        w.s1 = ws.second;
        w.i0 = (int)b->items.size();
        std::vector<std::pair<double, BatchItem>> flag, unocc;
        size_t soff = 0;
        for (int i = w.s0; i < w.s1; ++i) {
            const Problem &p = b->probs[i];
            const StateGeom &s = g[i];
            const double tile_cost = (double)p.nc;
            for (int c = 0; c < nchunk; ++c) {
                for (int band = 0; band < (s.tiles_f ? p.nv : 0); ++band)
                    for (int r = 0; r < s.rows_f; ++r)
                        flag.push_back({tile_cost * (mixed ? 1.5 : 1.25),
                                        BatchItem{i, 0, r, band, c, (int)(band * s.rows_f + r)}});
                const long long bt = s.tiles_n ? s.tiles_n / s.rows_n : 0;
                for (long long t = 0; t < bt; ++t)
                    for (int r = 0; r < s.rows_n; ++r)
                        unocc.push_back({tile_cost, BatchItem{i, 1, r, (int)t, c,
                                                              (int)(s.tiles_f + t * s.rows_n + r)}});
            }
            w.split_off.push_back(soff);
            soff += s.split;
        }
        w.split_bytes = soff;
        auto by_cost = [](const std::pair<double, BatchItem> &a, const std::pair<double, BatchItem> &c) {
            return a.first > c.first;
        };
        std::stable_sort(flag.begin(), flag.end(), by_cost);
        std::stable_sort(unocc.begin(), unocc.end(), by_cost);
        for (auto &f : flag) b->items.push_back(f.second);
        w.i_mid = (int)b->items.size();
        for (auto &u : unocc) b->items.push_back(u.second);
        w.i1 = (int)b->items.size();
        b->waves.push_back(w);
    }
    const size_t off_items = reserve(sizeof(BatchItem) * b->items.size());
    // Reduction jobs.
    for (int i = 0; i < nstates; ++i) {
        const StateGeom &s = g[i];
        const Problem &p = b->probs[i];
        b->jobs.push_back({nullptr, s.ach_seg, (int)s.ach_seg, nw,
                           reinterpret_cast<double2 *>(outs[i].achtemp), 0});
        b->jobs.push_back({nullptr, s.tiles_f, (int)s.tiles_f, nw,
                           reinterpret_cast<double2 *>(outs[i].asxtemp), 0});
        if (s.off_n1 || (outs[i].acht_n1_loc && p.nb > 0))
            b->jobs.push_back({nullptr, s.n1_seg, (int)s.n1_seg, p.nb,
                               reinterpret_cast<double2 *>(outs[i].acht_n1_loc), 0});
        if (s.achs_blocks)
            b->jobs.push_back({nullptr, s.achs_blocks, s.achs_blocks, 1,
                               reinterpret_cast<double2 *>(outs[i].achstemp), 0});
    }
    const size_t off_jobs = reserve(sizeof(ReduceJob) * b->jobs.size());
    const size_t off_prefix = reserve(sizeof(int) * (b->jobs.size() + 1));
    const size_t off_split = reserve(mixed ? max_wave : 0);
    b->dev_bytes = off;

    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaMalloc(&b->dev, b->dev_bytes);
    if (e != cudaSuccess) return set_error(e == cudaErrorMemoryAllocation ? GPP_ERR_OUT_OF_MEMORY : GPP_ERR_CUDA, cudaGetErrorString(e));
    char *d = b->dev;
    b->d_probs = reinterpret_cast<Problem *>(d + off_probs);
    b->d_parts = reinterpret_cast<Partials *>(d + off_parts);
    b->d_splits = reinterpret_cast<SplitPlanes *>(d + off_splits);
    b->d_items = reinterpret_cast<BatchItem *>(d + off_items);
    b->d_jobs = reinterpret_cast<ReduceJob *>(d + off_jobs);
    b->d_prefix = reinterpret_cast<int *>(d + off_prefix);
    b->d_heads = reinterpret_cast<int *>(d + off_heads);
    b->d_split = d + off_split;

    // Per-state partial pointers (the fault word is filled in by
    // upload_tables), split planes and reduction sources.
    size_t ji = 0;
    for (int i = 0; i < nstates; ++i) {
        const StateGeom &s = g[i];
        Partials part{};
        part.ach = reinterpret_cast<double2 *>(d + s.off_ach);
        part.ach_seg = s.ach_seg;
        part.ach_tile0 = 0;
        part.asx = reinterpret_cast<double2 *>(d + s.off_asx);
        part.asx_seg = s.tiles_f;
        part.n1 = s.off_n1 ? reinterpret_cast<double2 *>(d + s.off_n1) : nullptr;
        part.n1_seg = (int)s.n1_seg;
        part.err = nullptr;
        b->parts.push_back(part);
        if (part.n1 && s.rows_f != s.rows_n)  // shorter per-band segments are zero-padded
            b->n1_zero.push_back({part.n1, sizeof(double2) * (size_t)(s.n1_seg * b->probs[i].nb)});
        b->jobs[ji++].src = part.ach;
        b->jobs[ji++].src = part.asx;
        if (s.off_n1 || (outs[i].acht_n1_loc && b->probs[i].nb > 0)) {
            if (!part.n1) return set_error(GPP_ERR_UNSUPPORTED, "acht_n1_loc with no rows");
            b->jobs[ji++].src = part.n1;
        }
        if (s.achs_blocks) {
            b->achs.push_back({i, reinterpret_cast<double2 *>(d + s.off_achs)});
            b->achs_blocks.push_back(s.achs_blocks);
            b->jobs[ji++].src = reinterpret_cast<double2 *>(d + s.off_achs);
        }
    }
    b->splits.resize(nstates);
    for (auto &w : b->waves)
        for (int i = w.s0; i < w.s1; ++i)
            b->splits[i] = mixed ? split_planes_at(b->probs[i], b->d_split + w.split_off[i - w.s0])
                                 : SplitPlanes{};
    b->seg_prefix.push_back(0);
    for (auto &j : b->jobs) b->seg_prefix.push_back(b->seg_prefix.back() + j.nseg);
    b->total_segs = b->seg_prefix.back();
    return GPP_OK;
}

gpp_status upload_tables(gpp_batch *b, int *fault_word) {
    for (auto &p : b->parts) p.err = fault_word;
    b->err = fault_word;
    cudaError_t e = cudaMemcpy(b->d_probs, b->probs.data(), sizeof(Problem) * b->nstates,
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_parts, b->parts.data(), sizeof(Partials) * b->nstates,
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_splits, b->splits.data(), sizeof(SplitPlanes) * b->nstates,
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !b->items.empty())
        e = cudaMemcpy(b->d_items, b->items.data(), sizeof(BatchItem) * b->items.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !b->jobs.empty())
        e = cudaMemcpy(b->d_jobs, b->jobs.data(), sizeof(ReduceJob) * b->jobs.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_prefix, b->seg_prefix.data(), sizeof(int) * b->seg_prefix.size(),
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
    return GPP_OK;
}

// Launch configuration of the persistent kernels for a frequency chunk NWC:
// dynamic shared memory (opted in here, outside any stream capture) and the
// resident grid sizes.
template <int NWC>
cudaError_t prepare_persistent(gpp_batch *b) {
    if (b->precision == GPP_PRECISION_MIXED) {
        constexpr int RG = 2;  // one row pair of the split planes
        b->smem = sizeof(float4) * 2 * (2 * RG + b->warps) * batch_kc<NWC>();
        cudaError_t e = cudaSuccess;
        if constexpr (NWC == 3 || NWC == 8) {
            if (b->warps == 8) {
                auto kern8 = batched_noflag_mixed_kernel<RG, NWC, 8>;
                e = cudaFuncSetAttribute(kern8, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)b->smem);
                if (e != cudaSuccess) return e;
                b->grid = resident_blocks(kern8, b->smem, 256);
            }
        }
        if (b->warps == 4) {
            auto kern = batched_noflag_mixed_kernel<RG, NWC>;
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)b->smem);
            if (e != cudaSuccess) return e;
            b->grid = resident_blocks(kern, b->smem);
        }
        b->grid_flag = resident_blocks(batched_flag_mixed_kernel<NWC, 2>, 0);
    } else {
        constexpr int RN = NWC <= 4 ? 4 : 2;
        b->smem = 0;
        b->grid = b->grid_flag = resident_blocks(batched_fp64_kernel<RN, 2, NWC>, 0);
    }
    return cudaGetLastError();
}

template <int NWC>
cudaError_t launch_persistent(gpp_batch *b, int wave, cudaStream_t s) {
    const auto &w = b->waves[wave];
    int *heads = b->d_heads + 2 * wave;
    cudaError_t e = cudaSuccess;
    if (b->precision == GPP_PRECISION_MIXED) {
        constexpr int RG = 2;  // one row pair of the split planes
        const int nf = w.i_mid - w.i0, nu = w.i1 - w.i_mid;
        if (nf > 0) {
            batched_flag_mixed_kernel<NWC, 2><<<std::min(nf, b->grid_flag), kThreads, 0, s>>>(
                b->d_probs, b->d_parts, b->d_splits, b->d_items + w.i0, nf, heads);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && nu > 0) {
            bool done = false;
            if constexpr (NWC == 3 || NWC == 8) {
                if (b->warps == 8) {
                    batched_noflag_mixed_kernel<RG, NWC, 8><<<std::min(nu, b->grid), 256, b->smem,
                                                              s>>>(
                        b->d_probs, b->d_parts, b->d_splits, b->d_items + w.i_mid, nu, heads + 1);
                    done = true;
                }
            }
            if (!done)
                batched_noflag_mixed_kernel<RG, NWC><<<std::min(nu, b->grid), kThreads, b->smem,
                                                       s>>>(
                    b->d_probs, b->d_parts, b->d_splits, b->d_items + w.i_mid, nu, heads + 1);
            e = cudaGetLastError();
        }
    } else {
        constexpr int RN = NWC <= 4 ? 4 : 2;
        const int n = w.i1 - w.i0;
        if (n > 0) {
            batched_fp64_kernel<RN, 2, NWC><<<std::min(n, b->grid), kThreads, 0, s>>>(
                b->d_probs, b->d_parts, b->d_items + w.i0, n, heads);
            e = cudaGetLastError();
        }
    }
    return e;
}

cudaError_t prepare(gpp_batch *b) {
    switch (b->nw <= 4 ? b->nw : 8) {
        case 1: return prepare_persistent<1>(b);
        case 2: return prepare_persistent<2>(b);
        case 3: return prepare_persistent<3>(b);
        case 4: return prepare_persistent<4>(b);
        default: return prepare_persistent<8>(b);
    }
}

// Enqueue one full run of the batch on stream s.
gpp_status enqueue(gpp_batch *b, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(b->d_heads, 0, sizeof(int) * 2 * b->waves.size(), s);
    for (size_t k = 0; k < b->n1_zero.size() && e == cudaSuccess; ++k)
        e = cudaMemsetAsync(b->n1_zero[k].first, 0, b->n1_zero[k].second, s);
    int launches = 0;
    const int nwc = b->nw <= 4 ? b->nw : 8;
    for (size_t wv = 0; wv < b->waves.size() && e == cudaSuccess; ++wv) {
        const auto &w = b->waves[wv];
        if (b->precision == GPP_PRECISION_MIXED)
            for (int i = w.s0; i < w.s1 && e == cudaSuccess; ++i) {
                const Problem &p = b->probs[i];
                if (p.nb > 0 && p.ng > 0) {
                    e = launch_split(p, b->d_split + w.split_off[i - w.s0], 0, p.nb, s);
                    launches += 2;
                }
            }
        if (e != cudaSuccess) break;
        switch (nwc) {
            case 1: e = launch_persistent<1>(b, (int)wv, s); break;
            case 2: e = launch_persistent<2>(b, (int)wv, s); break;
            case 3: e = launch_persistent<3>(b, (int)wv, s); break;
            case 4: e = launch_persistent<4>(b, (int)wv, s); break;
            default: e = launch_persistent<8>(b, (int)wv, s); break;
        }
        launches += 2;
    }
    for (size_t k = 0; k < b->achs.size() && e == cudaSuccess; ++k) {
        e = launch_achstemp(b->probs[b->achs[k].first], b->achs[k].second, b->err, s);
        ++launches;
    }
    if (e == cudaSuccess && b->total_segs > 0) {
        // Same tree width as the one-state reduction, so a state gives the
        // same bits alone or in a batch.
        batched_reduce_kernel<512><<<b->total_segs, 512, 0, s>>>(b->d_jobs, b->d_prefix,
                                                                 (int)b->jobs.size());
        e = cudaGetLastError();
        ++launches;
    }
    b->launches_per_run = launches;
    if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
    return GPP_OK;
}

size_t default_split_budget() {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return (size_t)16 << 30;
    return std::max((size_t)1 << 30, free_b / 4);
}

}  // namespace

extern "C" {

int *gpp_internal_fault_word(void);

gpp_status gpp_batch_create(gpp_batch **out, const gpp_problem *problems,
                            const gpp_outputs *outs, int nstates) {
    if (!out || nstates <= 0 || !problems || !outs)
        return set_error(GPP_ERR_INVALID_ARGUMENT, "bad batch arguments");
    *out = nullptr;
    int *fault = gpp_internal_fault_word();
    if (!fault) return set_error(GPP_ERR_CUDA, "could not set up the device fault word");
    gpp_batch *b = new gpp_batch();
    gpp_status st = plan_batch(b, problems, outs, nstates, default_split_budget());
    if (st == GPP_OK) st = upload_tables(b, fault);
    if (st == GPP_OK) {
        cudaError_t e = prepare(b);
        if (e != cudaSuccess) st = set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
    }
    if (st != GPP_OK) {
        if (b->dev) cudaFree(b->dev);
        delete b;
        return st;
    }
    *out = b;
    return GPP_OK;
}

gpp_status gpp_batch_run(gpp_batch *b, gpp_stream_t stream) {
    if (!b) return set_error(GPP_ERR_INVALID_ARGUMENT, "batch is NULL");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) {
        gpp_status st = enqueue(b, s);
        count_launch(b->launches_per_run);
        return st;
    }
    if (!b->graph) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
        gpp_status st = enqueue(b, s);
        e = cudaStreamEndCapture(s, &g);
        if (st != GPP_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaError_t e = cudaGraphLaunch(b->graph, s);
    if (e != cudaSuccess) return set_error(GPP_ERR_CUDA, cudaGetErrorString(e));
    count_launch(b->launches_per_run);
    return GPP_OK;
}

gpp_status gpp_batch_destroy(gpp_batch *b) {
    if (!b) return GPP_OK;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->dev) cudaFree(b->dev);  // waits for work that still uses it
    delete b;
    return GPP_OK;
}

gpp_status gpp_sigma_batched(const gpp_problem *problems, const gpp_outputs *outs, int nstates,
                             gpp_stream_t stream) {
    if (nstates < 0 || (nstates > 0 && (!problems || !outs)))
        return set_error(GPP_ERR_INVALID_ARGUMENT, "bad batch");
    if (nstates == 0) return GPP_OK;
    gpp_batch *b = nullptr;
    gpp_status st = gpp_batch_create(&b, problems, outs, nstates);
    if (st != GPP_OK) return st;
    st = enqueue(b, reinterpret_cast<cudaStream_t>(stream));
    count_launch(b->launches_per_run);
    cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
    gpp_batch_destroy(b);
    return st;
}

}  // extern "C"

/*
 * gpp_gb300.h -- C ABI of the GB300-native GPP sigma library (libgpp_gb300.so).
 *
 * The General Plasmon Pole (GPP) sigma reduction of the DOE-CSFG-hackathon
 * mini-app (BerkeleyGW kernel): for bands n1, local G' rows my_igp, G columns
 * ig and frequencies iw,
 *
 *   achtemp[iw] += sum_{n1,my_igp} vcoul[igp] * 0.5 * scht(n1,my_igp,iw)
 *   asxtemp[iw] += sum_{n1<nvband,my_igp} occ * vcoul[igp] * ssxt(n1,my_igp,iw)
 *
 * with scht/ssxt the ig sums of noflagOCC_solver / flagOCC_solver
 * (gppComplex_seq.cpp:107-150) and igp = min(inv_igp_index[my_igp], ncouls-1).
 *
 * Conventions shared by every entry point:
 *  - Complex arrays are interleaved {re, im} doubles (16 bytes), row-major:
 *    aqsmtemp/aqsntemp [number_bands][ncouls], I_eps_array/wtilde_array
 *    [ngpown][ncouls] (gppKerSeq.cpp:194-197).  gpp_complex has the layout of
 *    the reference's GPPComplex (GPPComplex.h:68, a double2) and of
 *    std::complex<double>.
 *  - Unless stated otherwise, pointers are DEVICE pointers owned by the
 *    caller (as in gppCudaVer.cpp:306-318) and launches are asynchronous on
 *    the given stream (NULL = legacy default stream, as the reference uses).
 *  - Every entry point returns a gpp_status and never exits the process.
 *  - Results are deterministic: no floating-point atomics; every sum runs in
 *    a fixed order, so repeated calls give bit-identical outputs.
 */
#ifndef GPP_GB300_H
#define GPP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPP_GB300_VERSION_MAJOR 1
#define GPP_GB300_VERSION_MINOR 0

typedef struct gpp_complex { double re, im; } gpp_complex;

/* cudaStream_t without pulling in CUDA headers (same underlying type). */
typedef struct CUstream_st *gpp_stream_t;

typedef enum gpp_status {
    GPP_OK = 0,
    GPP_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, overflow, bad enum */
    GPP_ERR_CUDA = 2,             /* a CUDA runtime call failed (gpp_last_error_message) */
    GPP_ERR_OUT_OF_MEMORY = 3,    /* workspace or staging allocation failed */
    GPP_ERR_UNSUPPORTED = 4,      /* option not available for these sizes */
    GPP_ERR_BAD_INDEX = 5,        /* device saw inv_igp_index < 0 or indinv out of range */
    GPP_ERR_NOT_READY = 6,        /* gpp_wait timed out; the work is still running */
    GPP_ERR_DEVICE_TIMEOUT = 7    /* a kernel's bounded wait gave up; that call's results are invalid */
} gpp_status;

typedef enum gpp_precision {
    GPP_PRECISION_FP64 = 0,  /* FP64 CUDA-core kernel (<= 1e-12 rel vs the reference) */
    GPP_PRECISION_MIXED = 1  /* float-float bulk, FP64 near the plasmon pole (<= 1e-8 rel) */
} gpp_precision;

typedef enum gpp_semantics {
    /* gppComplex_seq.cpp / GPPComplex.cu: ssx is zeroed when
     * |ssx| > 4|I_eps| and wx < 0 (gppComplex_seq.cpp:58-59). Default. */
    GPP_SEM_COMPLEX_SEQ = 0,
    /* gppKerSeq.cpp: the cutoff condition abs(wx) < 0 never holds (:60). */
    GPP_SEM_KERSEQ = 1
} gpp_semantics;

/* ------------------------------------------------------------------------
 * Drop-in entry points with the reference's argument lists.
 * They take the stream set by gpp_set_stream() (default: legacy stream),
 * use the band-independent wx_array[nend-nstart] of the reference, the
 * GPP_SEM_COMPLEX_SEQ semantics of GPPComplex.cu, FP64 arithmetic (unless
 * gpp_set_dropin_precision below selects mixed), and ADD
 * into the caller's output arrays (the reference accumulates with atomics
 * into caller-zeroed arrays, gppCudaVer.cpp:360-361,376-377).
 * ------------------------------------------------------------------------ */

/* Replaces gppKernelGPU, declared at GPPComplex.h:304 and never defined in
 * the reference.  No nvband argument: every band takes the unoccupied
 * (noflagOCC) path.  indinv may be NULL; when given (ncouls entries) the
 * clamped igp is remapped as igp = indinv[igp] (identity in every reference
 * workload).  Frequencies iw = nstart .. nend-1 use wx_array[iw - nstart];
 * achtemp_re/im are indexed by iw - nstart. */
gpp_status gpp_kernel_gpu(const gpp_complex *wtilde_array, const gpp_complex *aqsntemp,
                          const gpp_complex *aqsmtemp, const gpp_complex *I_eps_array,
                          int ncouls, int ngpown, int number_bands, const double *wx_array,
                          double *achtemp_re, double *achtemp_im, const double *vcoul,
                          int nstart, int nend, const int *indinv, const int *inv_igp_index);

/* Replaces d_till_nvband (GPPComplex.cu:406, declared GPPComplex.h:306):
 * occupied bands n1 < nvband, 3 frequencies.  Adds into achtemp_re/im[3],
 * asxtemp[3] and acht_n1_loc[n1] (iw = 2 column).  Deterministic where the
 * reference's asxtemp / acht_n1_loc updates race (GPPComplex.cu:239,247). */
gpp_status gpp_till_nvband(int nvband, int ngpown, int ncouls, const int *inv_igp_index,
                           const double *wx_array, const gpp_complex *wtilde_array,
                           const gpp_complex *aqsmtemp, const gpp_complex *aqsntemp,
                           const gpp_complex *I_eps_array, gpp_complex *asxtemp,
                           const double *vcoul, gpp_complex *acht_n1_loc, double *achtemp_re,
                           double *achtemp_im, double occ);

/* Replaces d_noFlagOCCSolver (GPPComplex.cu:422, declared GPPComplex.h:310):
 * unoccupied bands nvband <= n1 < number_bands, 3 frequencies.  Adds into
 * achtemp_re/im[3] and acht_n1_loc[n1]. */
gpp_status gpp_noflag_occ_solver(int number_bands, int nvband, int ngpown, int ncouls,
                                 const int *inv_igp_index, const double *wx_array,
                                 const gpp_complex *wtilde_array, const gpp_complex *aqsmtemp,
                                 const gpp_complex *aqsntemp, const gpp_complex *I_eps_array,
                                 const double *vcoul, double *achtemp_re, double *achtemp_im,
                                 gpp_complex *acht_n1_loc);

/* Replaces the host-side reduce_achstemp loop of gppCudaVer.cpp:385-386
 * (gppKerSeq.cpp:67-100; d_reduce_achstemp is declared at GPPComplex.h:308
 * but never defined): the static COHSEX term over all bands, ADDED into
 * achstemp[0]. */
gpp_status gpp_reduce_achstemp(int number_bands, const int *inv_igp_index, int ncouls,
                               const gpp_complex *aqsmtemp, const gpp_complex *aqsntemp,
                               const gpp_complex *I_eps_array, gpp_complex *achstemp,
                               int ngpown, const double *vcoul);
/* The same static term with the reference's split destination: d_reduce_achstemp
 * (GPPComplex.h:308) takes double *achstemp_re, double *achstemp_im; the sum is
 * ADDED into achstemp_re[0] / achstemp_im[0]. */
gpp_status gpp_reduce_achstemp_split(int number_bands, const int *inv_igp_index, int ncouls,
                                     const gpp_complex *aqsmtemp, const gpp_complex *aqsntemp,
                                     const gpp_complex *I_eps_array, double *achstemp_re,
                                     double *achstemp_im, int ngpown, const double *vcoul);

/* Stream used by the drop-in entry points above (per host thread). */
gpp_status gpp_set_stream(gpp_stream_t stream);
gpp_stream_t gpp_get_stream(void);

/* No counterpart in the reference.  Arithmetic of the drop-in entry points
 * above except gpp_reduce_achstemp (per host thread): GPP_PRECISION_FP64
 * (the reference's) or GPP_PRECISION_MIXED (float-float, <= 1e-8 of FP64,
 * about 4x faster for the reference's call sequence); -1 restores the
 * process default, which is
 * GPP_PRECISION_MIXED when the environment has GPP_DROPIN_PRECISION=mixed
 * and GPP_PRECISION_FP64 otherwise -- so an unmodified reference driver can
 * run the mixed kernels.  gpp_get_dropin_precision returns the value in
 * effect. */
gpp_status gpp_set_dropin_precision(int precision);
int gpp_get_dropin_precision(void);

/* No counterpart in the reference.  How calls with band-independent
 * frequencies (wx_stride == 0: the drop-in entry points and gpp_sigma)
 * compute their unoccupied bands (per host thread): -1 (default) through
 * the band-sum GEMM when there are at least 32 unoccupied bands, 0 always
 * with the per-term kernel, 1 always through the GEMM, 2 as 1 with the FP64
 * GEMMs on the FP64 pipe instead of the tensor cores.  With wx the same
 * for every band the band sum factors out of the division:
 * achtemp[iw] = sum_{G',ig} M_iw G, G = sum_n1 c aqsn (one complex GEMM,
 * written in this library: in FP64 by default on the tensor cores, the
 * operands split into bf16 integer slices whose products the tensor cores
 * sum exactly (Ozaki scheme), with mode 2 as a 3M-form GEMM on the FP64
 * pipe; float-float on the FP32 pipes in mixed precision), several times
 * faster; the results agree with the per-term kernels to their rounding. */
gpp_status gpp_set_gemm_path(int mode);

/* ------------------------------------------------------------------------
 * Full problem API: occupied and unoccupied bands in one call, per-band
 * frequencies, asxtemp, precision and semantics selection.
 * ------------------------------------------------------------------------ */

typedef struct gpp_problem {
    int number_bands, nvband, ncouls, ngpown, nw;
    const gpp_complex *aqsmtemp;     /* [number_bands][ncouls] */
    const gpp_complex *aqsntemp;     /* [number_bands][ncouls] */
    const gpp_complex *I_eps_array;  /* [ngpown][ncouls] */
    const gpp_complex *wtilde_array; /* [ngpown][ncouls] */
    const double *vcoul;             /* [ncouls] */
    const int *inv_igp_index;        /* [ngpown]; values >= ncouls clamp to ncouls-1 */
    const int *indinv;               /* [ncouls] or NULL (see gpp_kernel_gpu) */
    const double *wx_array;          /* wx(n1,iw) = wx_array[n1*wx_stride + iw] */
    int wx_stride;                   /* 0: one [nw] row for all bands; >= nw: per band */
    double occ;                      /* occupation factor of asxtemp (reference: 1.0) */
    int semantics;                   /* gpp_semantics */
    int precision;                   /* gpp_precision */
} gpp_problem;

typedef struct gpp_outputs {
    gpp_complex *achtemp;     /* [nw], OVERWRITTEN (required) */
    gpp_complex *asxtemp;     /* [nw], OVERWRITTEN (required) */
    gpp_complex *acht_n1_loc; /* [number_bands] or NULL; needs nw >= 3 (iw = 2 column) */
    gpp_complex *achstemp;    /* [1] or NULL: static term of reduce_achstemp */
} gpp_outputs;

/* Device pointers in and out, asynchronous on `stream`.  Scratch memory comes
 * from a per-device workspace that the library grows on demand (the first
 * call at a larger size allocates; later calls do not). */
gpp_status gpp_sigma(const gpp_problem *problem, const gpp_outputs *out, gpp_stream_t stream);

/* Waits for `stream` (at most timeout_ms; < 0 waits forever) and reports
 * device-side faults of earlier gpp_sigma calls on this device: returns
 * GPP_ERR_DEVICE_TIMEOUT or GPP_ERR_BAD_INDEX once if a kernel gave up a
 * bounded wait or saw an invalid index (and clears the flag),
 * GPP_ERR_NOT_READY if the stream is still busy after timeout_ms. */
gpp_status gpp_wait(gpp_stream_t stream, int timeout_ms);

/* Host-memory convenience path (end-to-end): every array pointer in
 * `problem` is a HOST pointer, as are the outputs.  The call moves the inputs
 * to device buffers owned by `ctx` -- pinned (device-mapped) arrays by a
 * pull kernel on the SMs, overlapped with the computation in row pieces;
 * pageable ones, or all of them with GPP_HOST_PULL=ce in the environment, by
 * the copy engine -- runs gpp_sigma on the context's stream, copies results
 * back and returns when they are on the host.  Pinned memory is the fast
 * input: on GB300 the pull moves it at ~210 GB/s on every call, while
 * copy-engine copies were seen alternating with 10-40 GB/s calls. */
typedef struct gpp_context gpp_context;
gpp_status gpp_context_create(gpp_context **ctx);
gpp_status gpp_context_destroy(gpp_context *ctx);
gpp_status gpp_sigma_host(gpp_context *ctx, const gpp_problem *problem, const gpp_outputs *out);
/* Where the last gpp_sigma_host call on `ctx` spent its device time, from
 * CUDA events on the context's stream: host-to-device copies, gpp_sigma,
 * device-to-host copy (milliseconds; any pointer may be NULL). */
gpp_status gpp_context_last_timing(gpp_context *ctx, float *h2d_ms, float *compute_ms,
                                   float *d2h_ms);
/* The last call's timeline, milliseconds after its first copy began:
 * ms[0] = band arrays landed; then per row piece k, ms[1 + 2k] = the piece's
 * rows landed and ms[2 + 2k] = the kernels' stream reached the piece (a
 * piece whose start lies well after its landing was waiting on compute; the
 * reverse means compute waited on the copy).  *count receives 1 + 2 x pieces;
 * with capacity below it, only *count is set and GPP_ERR_INVALID_ARGUMENT
 * is returned. */
gpp_status gpp_context_last_trace(gpp_context *ctx, float *ms, int capacity, int *count);

/* No counterpart in the reference.  gpp_sigma for callers that cannot
 * allocate device memory -- applications that have handed the GPU's memory
 * to their own arena or to another runtime, or that cannot afford
 * cudaMalloc's device-wide synchronisation mid-step.  It always runs the
 * per-term FP64 kernels and keeps their block partials in a fixed 8 MiB array
 * in the library's device image (resident on every GPU that loads the
 * library), so it allocates nothing.  With per-band wx (wx_stride > 0), or
 * fewer than 32 unoccupied bands, those are gpp_sigma's own kernels and the
 * results are bit-identical; with band-independent wx and 32 or more
 * unoccupied bands gpp_sigma sums the bands as a GEMM instead, and the two
 * agree to FP64 rounding (1e-12 relative), not bit for bit, the per-term
 * kernels being the slower of the two there.  The argument checks and grid
 * limits are gpp_sigma's.  FP64 only; achtemp and asxtemp only (acht_n1_loc
 * and achstemp must be NULL); problems needing more than 8 MiB of partials
 * (the production shape needs ~5 MiB) return GPP_ERR_UNSUPPORTED.  All calls
 * share the array: calls whose GPU work overlaps in time race, so serialise
 * them on one stream.  The first call on a device looks up the array's
 * address; make it before any stream capture. */
gpp_status gpp_sigma_static_scratch(const gpp_problem *problem, const gpp_outputs *out,
                                    gpp_stream_t stream);

/* ------------------------------------------------------------------------
 * Batched states: many independent quasiparticle states (uneven sizes) in
 * one persistent launch over a work queue of (state, band tile, row tile).
 * ------------------------------------------------------------------------ */
/* One-shot: plans, runs and frees a batch on `stream`; returns when the
 * results are written.  All problems must share precision, nw and
 * semantics; outputs are overwritten as in gpp_sigma. */
gpp_status gpp_sigma_batched(const gpp_problem *problems, const gpp_outputs *outs, int nstates,
                             gpp_stream_t stream);

/* Reusable plan: the work list, device tables and scratch are built once
 * (gpp_batch_create allocates; the arrays behind the problems' pointers may
 * change contents between runs but not move).  gpp_batch_run enqueues a run
 * on `stream`; on a stream other than the legacy/per-thread default the
 * first run is captured into a CUDA graph and later runs replay it.
 * gpp_batch_destroy waits for outstanding runs and frees the plan. */
typedef struct gpp_batch gpp_batch;
gpp_status gpp_batch_create(gpp_batch **batch, const gpp_problem *problems,
                            const gpp_outputs *outs, int nstates);
gpp_status gpp_batch_run(gpp_batch *batch, gpp_stream_t stream);
gpp_status gpp_batch_destroy(gpp_batch *batch);

/* ------------------------------------------------------------------------
 * Autotuner for the mixed-precision unoccupied-band kernel.  It is compiled
 * in a few pipeline variants (shared-memory chunk width, stage count, block
 * barrier vs mbarrier ring).  gpp_autotune times every variant on `problem`
 * (its first max_bands unoccupied bands; 0 = all) on `stream`, keeps the
 * fastest for problems with the same frequency chunk on the current device,
 * and writes the choice to the file named by the GPP_TUNE_CACHE environment
 * variable, if set (read back on first use).  gpp_set_variant overrides the
 * choice (-1 restores the default); gpp_tuned_variant reports it.
 * ------------------------------------------------------------------------ */
gpp_status gpp_autotune(const gpp_problem *problem, int max_bands, gpp_stream_t stream,
                        int *best_variant);
gpp_status gpp_set_variant(int nw, int variant);
gpp_status gpp_tuned_variant(int nw, int *variant);
int gpp_variant_count(void);
const char *gpp_variant_name(int variant);

/* ------------------------------------------------------------------------
 * Introspection and measurement support.
 * ------------------------------------------------------------------------ */

/* Message of the last failing call on this host thread ("" if none). */
const char *gpp_last_error_message(void);

/* Number of kernel launches issued by this library on this host thread
 * since the last reset (for launch accounting in benchmarks). */
unsigned long long gpp_launch_count(void);
void gpp_reset_launch_count(void);

/* Kernel timing hook: when enabled, gpp_sigma records CUDA events around
 * its dominant kernel on the launching stream; gpp_last_kernel_ms returns
 * the elapsed milliseconds of the most recent call (synchronises on the
 * end event). */
gpp_status gpp_enable_kernel_timing(int enable);
gpp_status gpp_last_kernel_ms(float *ms);

/* Measured FP64 / FP32 fused multiply-add peaks of the current device in
 * TFLOP/s (FMA = 2 flops), from a short dependent-chain-free probe kernel. */
gpp_status gpp_probe_fma_peaks(double *fp64_tflops, double *fp32_tflops);

/* No counterpart in the reference.  Failure-path self-test: launches one
 * block on `stream` that waits on a shared-memory barrier nothing will
 * complete, gives up after `polls` polls (1 .. 1<<22) exactly as the mixed
 * kernels' pipeline waits do, and records the timeout in the device fault
 * word.  The next gpp_wait on that stream returns GPP_ERR_DEVICE_TIMEOUT
 * once; the context stays usable. */
gpp_status gpp_selftest_wait_timeout(int polls, gpp_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* GPP_GB300_H */

/*
 * GPP sigma oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference's CPU algorithm for the
 * BerkeleyGW General Plasmon Pole sigma reduction (DOE-CSFG-hackathon).
 * Only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark load this library, and only as the checker or as the timed CPU
 * baseline.  The CUDA product path never calls into it.
 *
 * Parity is pinned: the restatement reproduces the reference's published
 * known answers (README.md:25-42, ramp inputs of gppKerSeq.cpp:225-258)
 * digit for digit, and matches the reference's own functions, compiled from
 * gppComplex_seq.cpp / gppKerSeq.cpp by oracle/build_oracle.py, bit for bit
 * on seeded inputs (tests/golden/).
 */
#ifndef GPP_ORACLE_H
#define GPP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* 16-byte interleaved {re, im}: the layout of GPPComplex (Complex.h:15-18),
 * double2 (GPPComplex.h:68) and std::complex<double>. */
typedef struct { double re, im; } oracle_complex;

/* Semantics of the two sequential references.
 *  COMPLEX_SEQ: gppComplex_seq.cpp -- ssx cutoff fires when wx < 0
 *               (gppComplex_seq.cpp:58-59), |z| = sqrt(re^2+im^2).
 *  KERSEQ:      gppKerSeq.cpp -- cutoff condition abs(wx) < 0 never holds
 *               (gppKerSeq.cpp:59-60), std::complex product order. */
enum { ORACLE_SEM_COMPLEX_SEQ = 0, ORACLE_SEM_KERSEQ = 1 };

typedef struct {
    int number_bands, nvband, ncouls, ngpown, nw;
    const oracle_complex *aqsmtemp;     /* [number_bands][ncouls] */
    const oracle_complex *aqsntemp;     /* [number_bands][ncouls] */
    const oracle_complex *I_eps_array;  /* [ngpown][ncouls] */
    const oracle_complex *wtilde_array; /* [ngpown][ncouls] */
    const double *vcoul;                /* [ncouls] */
    const int *inv_igp_index;           /* [ngpown] */
    const double *wx_array;             /* wx(n1,iw) = wx_array[n1*wx_stride + iw] */
    int wx_stride;                      /* 0: band-independent [nw]; >= nw: per band */
    double occ;
    int semantics;
    int band_begin, band_end;           /* bands actually summed; [0, number_bands) for the full sum */
} oracle_problem;

typedef struct {
    oracle_complex *achtemp;      /* [nw] (required) */
    oracle_complex *asxtemp;      /* [nw] (required) */
    oracle_complex *acht_n1_loc;  /* [number_bands] or NULL; needs nw >= 3 (uses iw = 2) */
    oracle_complex *achstemp;     /* [1] or NULL: the static term of reduce_achstemp */
} oracle_outputs;

/* Sum in the reference's sequential order (n1 outer, my_igp inner).  With
 * nthreads > 1 the per-(n1, my_igp) contributions are computed in parallel
 * and then added in that same order, so the result is bit-identical to
 * nthreads == 1.  Returns 0 on success, -1 on invalid arguments, -2 if out
 * of host memory. */
int oracle_sigma(const oracle_problem *p, oracle_outputs *out, int nthreads);

/* The reference's OpenMP loop shape (gppOpenMP3.cpp:278-333): the same
 * per-(n1, my_igp) work, spread over nthreads host threads with dynamic
 * scheduling, per-thread partial sums combined at the end.  Used as the
 * timed CPU baseline; the summation order depends on the thread count. */
int oracle_sigma_omp(const oracle_problem *p, oracle_outputs *out, int nthreads);

/* Ramp inputs of gppKerSeq.cpp:225-258 (the README known-answer inputs):
 * aqs*, I_eps, wtilde = (i+j)(0.5+0.5i); vcoul[i] = i;
 * inv_igp_index[i] = (i+1)*ncouls/ngpown; wx[iw] = e_lk - e_n1kq + dw*(iw-1)
 * with the |wx| < to1 clamp of gppKerSeq.cpp:257. */
void oracle_ramp_inputs(int number_bands, int ncouls, int ngpown, int nw,
                        oracle_complex *aqsmtemp, oracle_complex *aqsntemp,
                        oracle_complex *I_eps_array, oracle_complex *wtilde_array,
                        double *vcoul, int *inv_igp_index, double *wx_array);

/* The same sums evaluated in long double (64-bit significand on x86-64,
 * 113-bit on aarch64) with Neumaier-compensated accumulation: a reference
 * value to measure the rounding error of the FP64 and GPU paths against.
 * It follows the reference's algebra and branches but not its operation
 * order, so it is not bit-comparable with the reference.  Same return codes
 * as oracle_sigma. */
int oracle_sigma_extended(const oracle_problem *p, oracle_outputs *out, int nthreads);

int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif

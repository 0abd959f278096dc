/*
 * GPP sigma oracle -- TEST INFRASTRUCTURE ONLY (see gpp_oracle.h).
 *
 * Plain-C FP64 restatement of the reference's sequential GPP kernel.  Every
 * expression keeps the reference's operation order so that, compiled with
 * -ffp-contract=off, results are bit-identical to the reference's own
 * functions (checked in tests/test_oracle.py against fixtures produced by
 * the reference itself).
 *
 * Reference map (file:line in DOE-CSFG-hackathon):
 *   term_ssx_sch      ssxt_scht_solver   gppComplex_seq.cpp:16-63, gppKerSeq.cpp:18-64
 *   flag_row          flagOCC_solver     gppComplex_seq.cpp:107-128, gppKerSeq.cpp:106-124
 *   noflag_row        noflagOCC_solver   gppComplex_seq.cpp:131-150, gppKerSeq.cpp:127-145
 *   achstemp_row      reduce_achstemp    gppComplex_seq.cpp:66-101, gppKerSeq.cpp:67-100
 *   pair_contrib      loop body          gppComplex_seq.cpp:340-382, gppKerSeq.cpp:271-313
 *   oracle_sigma      driver loop nest   gppComplex_seq.cpp:335-383
 *   oracle_sigma_omp  OpenMP loop shape  gppOpenMP3.cpp:278-333
 *   oracle_ramp_inputs ramp init         gppKerSeq.cpp:225-258
 *   oracle_sigma_extended  the same sums in long double with compensated
 *                          accumulation: a reference value for measuring the
 *                          FP64 paths' own rounding (no operation-order parity)
 */
#include "gpp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef oracle_complex cx;

/* Constants of ssxt_scht_solver (gppComplex_seq.cpp:20-23). */
#define GPP_TO1 1e-6
#define GPP_SEXCUT 4.0
#define GPP_LIMITONE (1.0 / (GPP_TO1 * 4.0))
#define GPP_LIMITTWO 0.25 /* pow(0.5, 2) */

static inline cx mk(double re, double im) { cx z; z.re = re; z.im = im; return z; }
/* a*b with re = a.re*b.re - a.im*b.im, im = a.re*b.im + a.im*b.re
 * (GPPComplex_product, Complex.h:167-174; also GCC's std::complex product). */
static inline cx cmul(cx a, cx b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cconj(cx a) { return mk(a.re, -a.im); }
static inline cx cscale(cx a, double s) { return mk(a.re * s, a.im * s); }
static inline cx cadd(cx a, cx b) { return mk(a.re + b.re, a.im + b.im); }
/* |z|^2 as real(z*conj(z)): re*re - im*(-im). */
static inline double cnorm2(cx a) { return a.re * a.re - a.im * (-a.im); }

/* One (ig) term of the occupied-band solver: returns ssx and sch before the
 * matngmatmgp factor.  wt2 = wtilde^2, omega2 = wt2 * I_eps. */
static void term_ssx_sch(int sem, double wxt, cx wt, cx wt2, cx omega2, cx ieps,
                         cx *ssx_out, cx *sch_out)
{
    cx sch = mk(0.0, 0.0), ssx = mk(0.0, 0.0);
    cx wdiff = mk(wxt - wt.re, 0.0 - wt.im);
    double rden = 1.0 / cnorm2(wdiff);
    cx delw = cscale(cmul(wt, cconj(wdiff)), rden);
    double delwr = cnorm2(delw);
    double wdiffr = cnorm2(wdiff);

    if (wdiffr > GPP_LIMITTWO && delwr < GPP_LIMITONE) {
        sch = cmul(delw, ieps);
        double c = wxt * wxt;          /* pow(wxt, 2) */
        double r = 1.0 / (c * c);      /* 1 / pow(c, 2) */
        ssx = mk(omega2.re * c * r, omega2.im * c * r);
    } else if (delwr > GPP_TO1) {
        cx cden = cscale(cmul(wt2, mk(0.5 + delw.re, delw.im)), 4.0);
        double r = 1.0 / cnorm2(cden);
        cx neg_omega2 = mk(-omega2.re, -omega2.im);
        if (sem == ORACLE_SEM_KERSEQ) {
            /* -Omega2 * conj(cden) * rden * delw, left to right (gppKerSeq.cpp:51) */
            ssx = cmul(cscale(cmul(neg_omega2, cconj(cden)), r), delw);
        } else {
            /* (-Omega2 conj(cden)) (delw rden)  (gppComplex_seq.cpp:50) */
            ssx = cmul(cmul(neg_omega2, cconj(cden)), cscale(delw, r));
        }
    }

    if (sem == ORACLE_SEM_COMPLEX_SEQ) {
        /* gppComplex_seq.cpp:58-59: |ssx| > 4|I_eps| and wx < 0 zeroes ssx. */
        double cutoff = sqrt(ieps.re * ieps.re + ieps.im * ieps.im) * GPP_SEXCUT;
        if (sqrt(ssx.re * ssx.re + ssx.im * ssx.im) > cutoff && wxt < 0.0) ssx = mk(0.0, 0.0);
    }
    /* KERSEQ: the condition abs(wxt) < 0 is never true (gppKerSeq.cpp:60). */
    *ssx_out = ssx;
    *sch_out = sch;
}

static void flag_row(const oracle_problem *p, double wxt, int my_igp, int n1, int igp,
                     cx *ssxt, cx *scht)
{
    const int nc = p->ncouls;
    const cx *wrow = p->wtilde_array + (size_t)my_igp * nc;
    const cx *erow = p->I_eps_array + (size_t)my_igp * nc;
    const cx *nrow = p->aqsntemp + (size_t)n1 * nc;
    const cx mygpvar1 = cconj(p->aqsmtemp[(size_t)n1 * nc + igp]);
    for (int ig = 0; ig < nc; ++ig) {
        cx wt = wrow[ig];
        cx wt2 = mk(wt.re * wt.re - wt.im * wt.im, 2.0 * wt.re * wt.im);
        cx omega2 = cmul(wt2, erow[ig]);
        cx matng = cmul(nrow[ig], mygpvar1);
        cx ssx, sch;
        term_ssx_sch(p->semantics, wxt, wt, wt2, omega2, erow[ig], &ssx, &sch);
        *ssxt = cadd(*ssxt, cmul(matng, ssx));
        *scht = cadd(*scht, cmul(matng, sch));
    }
}

static cx noflag_row(const oracle_problem *p, double wxt, int my_igp, int n1, int igp)
{
    const int nc = p->ncouls;
    const cx *wrow = p->wtilde_array + (size_t)my_igp * nc;
    const cx *erow = p->I_eps_array + (size_t)my_igp * nc;
    const cx *nrow = p->aqsntemp + (size_t)n1 * nc;
    const cx mygpvar1 = cconj(p->aqsmtemp[(size_t)n1 * nc + igp]);
    cx acc = mk(0.0, 0.0);
    for (int ig = 0; ig < nc; ++ig) {
        cx wt = wrow[ig];
        cx wdiff = mk(wxt - wt.re, 0.0 - wt.im);
        double rden = 1.0 / cnorm2(wdiff);
        cx delw = cscale(cmul(wt, cconj(wdiff)), rden);
        if (p->semantics == ORACLE_SEM_KERSEQ) {
            /* ((mygpvar1 aqsn) delw) I_eps (gppKerSeq.cpp:141) */
            acc = cadd(acc, cmul(cmul(cmul(mygpvar1, nrow[ig]), delw), erow[ig]));
        } else {
            /* (mygpvar1 aqsn)(delw I_eps) (gppComplex_seq.cpp:146) */
            acc = cadd(acc, cmul(cmul(mygpvar1, nrow[ig]), cmul(delw, erow[ig])));
        }
    }
    return acc;
}

/* Per (n1, my_igp) static term (reduce_achstemp body, one my_igp). */
static cx achstemp_row(const oracle_problem *p, int n1, int my_igp, int igp)
{
    const int nc = p->ncouls;
    cx mygpvar1 = cconj(p->aqsmtemp[(size_t)n1 * nc + igp]);
    cx aqsn_igp = p->aqsntemp[(size_t)n1 * nc + igp];
    cx ie = p->I_eps_array[(size_t)my_igp * nc + igp];
    cx schs = mk(-ie.re, -ie.im);
    cx matng = cmul(aqsn_igp, mygpvar1);
    cx schstemp = mk(0.0, 0.0);
    double a = (p->semantics == ORACLE_SEM_KERSEQ) ? hypot(schs.re, schs.im)
                                                   : sqrt(schs.re * schs.re + schs.im * schs.im);
    if (a > GPP_TO1) schstemp = cadd(schstemp, cmul(matng, schs));
    return cscale(schstemp, p->vcoul[igp] * 0.5);
}

static inline int clamp_igp(const oracle_problem *p, int my_igp)
{
    int igp = p->inv_igp_index[my_igp];
    if (igp >= p->ncouls) igp = p->ncouls - 1; /* gppComplex_seq.cpp:342-344 */
    return igp;
}

/* Contribution of one (n1, my_igp) pair to achtemp[iw], asxtemp[iw] and
 * acht_n1_loc[n1] (iw = 2 column). */
static void pair_contrib(const oracle_problem *p, int n1, int my_igp,
                         cx *ach, cx *asx, cx *acht_n1)
{
    const int nw = p->nw;
    const int igp = clamp_igp(p, my_igp);
    const double v = p->vcoul[igp];
    const int flag_occ = n1 < p->nvband;
    for (int iw = 0; iw < nw; ++iw) {
        const double wxt = p->wx_array[(size_t)n1 * p->wx_stride + iw];
        cx sch_iw = mk(0.0, 0.0);
        asx[iw] = mk(0.0, 0.0);
        if (flag_occ) {
            cx ssxt = mk(0.0, 0.0), scht = mk(0.0, 0.0);
            flag_row(p, wxt, my_igp, n1, igp, &ssxt, &scht);
            sch_iw = cscale(scht, 0.5);
            if (p->semantics == ORACLE_SEM_KERSEQ)
                asx[iw] = cscale(cscale(ssxt, p->occ), v);  /* ssx * occ * vcoul */
            else
                asx[iw] = cscale(ssxt, p->occ * v);         /* mult(ssx, occ*vcoul) */
        } else {
            sch_iw = cscale(noflag_row(p, wxt, my_igp, n1, igp), 0.5);
        }
        ach[iw] = cscale(sch_iw, v);
        if (iw == 2) *acht_n1 = cscale(sch_iw, v);
    }
}

static int validate(const oracle_problem *p, const oracle_outputs *o)
{
    if (!p || !o || !o->achtemp || !o->asxtemp) return -1;
    if (p->number_bands < 0 || p->nvband < 0 || p->ncouls <= 0 || p->ngpown < 0 || p->nw <= 0) return -1;
    if (p->wx_stride != 0 && p->wx_stride < p->nw) return -1;
    if (p->band_begin < 0 || p->band_end > p->number_bands || p->band_begin > p->band_end) return -1;
    if (o->acht_n1_loc && p->nw < 3) return -1;
    for (int i = 0; i < p->ngpown; ++i)
        if (p->inv_igp_index[i] < 0) return -1;
    return 0;
}

static void zero_outputs(const oracle_problem *p, oracle_outputs *o)
{
    memset(o->achtemp, 0, sizeof(cx) * (size_t)p->nw);
    memset(o->asxtemp, 0, sizeof(cx) * (size_t)p->nw);
    if (o->acht_n1_loc) memset(o->acht_n1_loc, 0, sizeof(cx) * (size_t)p->number_bands);
    if (o->achstemp) o->achstemp[0] = mk(0.0, 0.0);
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_sigma(const oracle_problem *p, oracle_outputs *o, int nthreads)
{
    if (validate(p, o)) return -1;
    zero_outputs(p, o);
    const int nw = p->nw, ng = p->ngpown;
    const int nbands = p->band_end - p->band_begin;
    if (nbands == 0 || ng == 0) return 0;
    /* Per-pair contributions: [band][my_igp][nw] for ach and asx, plus the
     * iw = 2 column and the static term. */
    const size_t npairs = (size_t)nbands * (size_t)ng;
    cx *ach = (cx *)malloc(sizeof(cx) * npairs * (size_t)nw);
    cx *asx = (cx *)malloc(sizeof(cx) * npairs * (size_t)nw);
    cx *n1c = (cx *)malloc(sizeof(cx) * npairs);
    cx *sts = (cx *)malloc(sizeof(cx) * npairs);
    if (!ach || !asx || !n1c || !sts) { free(ach); free(asx); free(n1c); free(sts); return -2; }
    if (nthreads < 1) nthreads = 1;

#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long long pr = 0; pr < (long long)npairs; ++pr) {
        const int n1 = p->band_begin + (int)(pr / ng);
        const int my_igp = (int)(pr % ng);
        n1c[pr] = mk(0.0, 0.0);
        pair_contrib(p, n1, my_igp, ach + (size_t)pr * nw, asx + (size_t)pr * nw, &n1c[pr]);
        sts[pr] = achstemp_row(p, n1, my_igp, clamp_igp(p, my_igp));
    }

    /* Sequential accumulation in the reference's (n1, my_igp) order:
     * asxtemp inside the iw loop (gppComplex_seq.cpp:363), achtemp after it
     * (:378-379), acht_n1_loc (:381), achstemp via reduce_achstemp (:338). */
    for (size_t pr = 0; pr < npairs; ++pr) {
        const int n1 = p->band_begin + (int)(pr / ng);
        if (n1 < p->nvband)
            for (int iw = 0; iw < nw; ++iw) o->asxtemp[iw] = cadd(o->asxtemp[iw], asx[pr * nw + iw]);
        for (int iw = 0; iw < nw; ++iw) o->achtemp[iw] = cadd(o->achtemp[iw], ach[pr * nw + iw]);
        if (o->acht_n1_loc) o->acht_n1_loc[n1] = cadd(o->acht_n1_loc[n1], n1c[pr]);
        if (o->achstemp) o->achstemp[0] = cadd(o->achstemp[0], sts[pr]);
    }
    free(ach); free(asx); free(n1c); free(sts);
    return 0;
}

int oracle_sigma_omp(const oracle_problem *p, oracle_outputs *o, int nthreads)
{
    if (validate(p, o)) return -1;
    zero_outputs(p, o);
    const int nw = p->nw, ng = p->ngpown;
    if (nthreads < 1) nthreads = 1;
    /* Per thread: running achtemp/asxtemp partials, then ach/asx scratch. */
    const size_t per = (size_t)4 * nw;
    cx *part = (cx *)calloc((size_t)nthreads * per, sizeof(cx));
    if (!part) return -2;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        cx *acc_ach = part + (size_t)t * per;
        cx *acc_asx = acc_ach + nw;
        cx *ach = acc_asx + nw;
        cx *asx = ach + nw;
        for (int n1 = p->band_begin; n1 < p->band_end; ++n1) {
#ifdef _OPENMP
#pragma omp for schedule(dynamic) nowait
#endif
            for (int my_igp = 0; my_igp < ng; ++my_igp) {
                cx n1c = mk(0.0, 0.0);
                pair_contrib(p, n1, my_igp, ach, asx, &n1c);
                for (int iw = 0; iw < nw; ++iw) {
                    acc_ach[iw] = cadd(acc_ach[iw], ach[iw]);
                    if (n1 < p->nvband) acc_asx[iw] = cadd(acc_asx[iw], asx[iw]);
                }
            }
        }
    }
    for (int t = 0; t < nthreads; ++t)
        for (int iw = 0; iw < nw; ++iw) {
            o->achtemp[iw] = cadd(o->achtemp[iw], part[(size_t)t * per + iw]);
            o->asxtemp[iw] = cadd(o->asxtemp[iw], part[(size_t)t * per + nw + iw]);
        }
    free(part);
    return 0;
}

void oracle_ramp_inputs(int nb, int nc, int ng, int nw,
                        cx *aqsm, cx *aqsn, cx *ieps, cx *wt,
                        double *vcoul, int *inv_igp_index, double *wx)
{
    const cx expr = mk(0.5, 0.5);
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nc; ++j) {
            aqsn[(size_t)i * nc + j] = cscale(expr, (double)(i + j));
            aqsm[(size_t)i * nc + j] = cscale(expr, (double)(i + j));
        }
    for (int i = 0; i < ng; ++i) {
        for (int j = 0; j < nc; ++j) {
            ieps[(size_t)i * nc + j] = cscale(expr, (double)(i + j));
            wt[(size_t)i * nc + j] = cscale(expr, (double)(i + j));
        }
        inv_igp_index[i] = (i + 1) * nc / ng;
    }
    for (int i = 0; i < nc; ++i) vcoul[i] = 1.0 * i;
    const double e_lk = 10.0, dw = 1.0, e_n1kq = 6.0;
    for (int iw = 0; iw < nw; ++iw) {
        wx[iw] = e_lk - e_n1kq + dw * ((iw + 1) - 2);
        if (fabs(wx[iw]) < GPP_TO1) wx[iw] = GPP_TO1;
    }
}

/* ------------------------------------------------------------------------
 * Extended-precision reference: the algebra of the functions above (same
 * branches, cutoff and semantics), evaluated in long double -- 64-bit
 * significand on x86-64, 113-bit on aarch64 -- with Neumaier-compensated
 * sums over ig and over the (n1, my_igp) pairs.  It does not follow the
 * reference's operation order; it serves as the "true" value against which
 * both the FP64 oracle and the GPU paths show their rounding error.  Branch
 * decisions can differ from FP64 only for terms within rounding distance of
 * a threshold.
 */
typedef long double ld;
typedef struct { ld re, im; } cxl;
typedef struct { ld s, c; } ksum; /* Neumaier running sum: s + c */

static inline cxl mkl(ld re, ld im) { cxl z; z.re = re; z.im = im; return z; }
static inline cxl cxl_of(cx a) { return mkl(a.re, a.im); }
static inline cxl mull(cxl a, cxl b) { return mkl(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cxl conjl_(cxl a) { return mkl(a.re, -a.im); }
static inline cxl scalel(cxl a, ld s) { return mkl(a.re * s, a.im * s); }
static inline ld norm2l(cxl a) { return a.re * a.re + a.im * a.im; }
static inline void kadd(ksum *k, ld x)
{
    const ld t = k->s + x;
    if (fabsl(k->s) >= fabsl(x)) k->c += (k->s - t) + x;
    else k->c += (x - t) + k->s;
    k->s = t;
}
static inline ld kval(const ksum *k) { return k->s + k->c; }

static void term_l(int sem, ld wxt, cxl wt, cxl ieps, cxl *ssx_out, cxl *sch_out)
{
    cxl sch = mkl(0, 0), ssx = mkl(0, 0);
    const cxl wt2 = mull(wt, wt), omega2 = mull(wt2, ieps);
    const cxl wdiff = mkl(wxt - wt.re, -wt.im);
    const ld rden = 1.0L / norm2l(wdiff);
    const cxl delw = scalel(mull(wt, conjl_(wdiff)), rden);
    const ld delwr = norm2l(delw), wdiffr = norm2l(wdiff);
    if (wdiffr > (ld)GPP_LIMITTWO && delwr < (ld)GPP_LIMITONE) {
        sch = mull(delw, ieps);
        ssx = scalel(omega2, 1.0L / (wxt * wxt));
    } else if (delwr > (ld)GPP_TO1) {
        const cxl cden = scalel(mull(wt2, mkl(0.5L + delw.re, delw.im)), 4.0L);
        const cxl t = mull(mkl(-omega2.re, -omega2.im), conjl_(cden));
        ssx = mull(t, scalel(delw, 1.0L / norm2l(cden)));
    }
    if (sem == ORACLE_SEM_COMPLEX_SEQ && wxt < 0 && sqrtl(norm2l(ssx)) > sqrtl(norm2l(ieps)) * 4.0L)
        ssx = mkl(0, 0);
    *ssx_out = ssx;
    *sch_out = sch;
}

/* Per (n1, my_igp, iw): compensated sums of the ig terms. */
static void pair_l(const oracle_problem *p, int n1, int my_igp, int iw, cxl *sch, cxl *ssx)
{
    const int nc = p->ncouls;
    const cx *wrow = p->wtilde_array + (size_t)my_igp * nc;
    const cx *erow = p->I_eps_array + (size_t)my_igp * nc;
    const cx *nrow = p->aqsntemp + (size_t)n1 * nc;
    const int igp = clamp_igp(p, my_igp);
    const cxl m = conjl_(cxl_of(p->aqsmtemp[(size_t)n1 * nc + igp]));
    const ld wxt = p->wx_array[(size_t)n1 * p->wx_stride + iw];
    ksum hr = {0, 0}, hi = {0, 0}, xr = {0, 0}, xi = {0, 0};
    for (int ig = 0; ig < nc; ++ig) {
        const cxl wt = cxl_of(wrow[ig]), ie = cxl_of(erow[ig]);
        const cxl matng = mull(cxl_of(nrow[ig]), m);
        if (n1 < p->nvband) {
            cxl x, h;
            term_l(p->semantics, wxt, wt, ie, &x, &h);
            const cxl a = mull(matng, h), b = mull(matng, x);
            kadd(&hr, a.re); kadd(&hi, a.im); kadd(&xr, b.re); kadd(&xi, b.im);
        } else {
            const cxl wdiff = mkl(wxt - wt.re, -wt.im);
            const cxl delw = scalel(mull(wt, conjl_(wdiff)), 1.0L / norm2l(wdiff));
            const cxl a = mull(matng, mull(delw, ie));
            kadd(&hr, a.re); kadd(&hi, a.im);
        }
    }
    *sch = mkl(kval(&hr), kval(&hi));
    *ssx = mkl(kval(&xr), kval(&xi));
}

int oracle_sigma_extended(const oracle_problem *p, oracle_outputs *o, int nthreads)
{
    if (validate(p, o)) return -1;
    zero_outputs(p, o);
    const int nw = p->nw, ng = p->ngpown;
    const int nbands = p->band_end - p->band_begin;
    if (nbands == 0 || ng == 0) return 0;
    const size_t npairs = (size_t)nbands * (size_t)ng;
    /* Per pair and frequency: ach re/im, asx re/im; per pair: static term. */
    ld *v = (ld *)malloc(sizeof(ld) * npairs * ((size_t)nw * 4 + 2));
    if (!v) return -2;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long long pr = 0; pr < (long long)npairs; ++pr) {
        const int n1 = p->band_begin + (int)(pr / ng);
        const int my_igp = (int)(pr % ng);
        const int igp = clamp_igp(p, my_igp);
        const ld vc = p->vcoul[igp];
        ld *row = v + (size_t)pr * ((size_t)nw * 4 + 2);
        for (int iw = 0; iw < nw; ++iw) {
            cxl sch, ssx;
            pair_l(p, n1, my_igp, iw, &sch, &ssx);
            row[4 * iw + 0] = sch.re * 0.5L * vc;
            row[4 * iw + 1] = sch.im * 0.5L * vc;
            row[4 * iw + 2] = ssx.re * (ld)p->occ * vc;
            row[4 * iw + 3] = ssx.im * (ld)p->occ * vc;
        }
        /* static term (achstemp_row) */
        const int nc = p->ncouls;
        const cxl m = conjl_(cxl_of(p->aqsmtemp[(size_t)n1 * nc + igp]));
        const cxl ie = cxl_of(p->I_eps_array[(size_t)my_igp * nc + igp]);
        const cxl schs = mkl(-ie.re, -ie.im);
        cxl st = mkl(0, 0);
        if (sqrtl(norm2l(schs)) > (ld)GPP_TO1)
            st = scalel(mull(mull(cxl_of(p->aqsntemp[(size_t)n1 * nc + igp]), m), schs), vc * 0.5L);
        row[4 * nw] = st.re;
        row[4 * nw + 1] = st.im;
    }
    for (int iw = 0; iw < nw; ++iw) {
        ksum ar = {0, 0}, ai = {0, 0}, xr = {0, 0}, xi = {0, 0};
        for (size_t pr = 0; pr < npairs; ++pr) {
            const ld *row = v + pr * ((size_t)nw * 4 + 2);
            kadd(&ar, row[4 * iw]); kadd(&ai, row[4 * iw + 1]);
            if (p->band_begin + (int)(pr / ng) < p->nvband) {
                kadd(&xr, row[4 * iw + 2]); kadd(&xi, row[4 * iw + 3]);
            }
        }
        o->achtemp[iw] = mk((double)kval(&ar), (double)kval(&ai));
        o->asxtemp[iw] = mk((double)kval(&xr), (double)kval(&xi));
    }
    if (o->acht_n1_loc && nw >= 3)
        for (int n1 = p->band_begin; n1 < p->band_end; ++n1) {
            ksum ar = {0, 0}, ai = {0, 0};
            for (int g = 0; g < ng; ++g) {
                const ld *row = v + ((size_t)(n1 - p->band_begin) * ng + g) * ((size_t)nw * 4 + 2);
                kadd(&ar, row[8]); kadd(&ai, row[9]);
            }
            o->acht_n1_loc[n1] = mk((double)kval(&ar), (double)kval(&ai));
        }
    if (o->achstemp) {
        ksum ar = {0, 0}, ai = {0, 0};
        for (size_t pr = 0; pr < npairs; ++pr) {
            const ld *row = v + pr * ((size_t)nw * 4 + 2);
            kadd(&ar, row[4 * nw]); kadd(&ai, row[4 * nw + 1]);
        }
        o->achstemp[0] = mk((double)kval(&ar), (double)kval(&ai));
    }
    free(v);
    return 0;
}

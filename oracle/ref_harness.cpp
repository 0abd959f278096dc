/*
 * Harness around the reference's OWN sequential GPP functions -- TEST
 * INFRASTRUCTURE ONLY.
 *
 * oracle/build_oracle.py compiles this file together with the unmodified
 * reference source (gppComplex_seq.cpp with REF_COMPLEX_SEQ, gppKerSeq.cpp
 * with REF_KERSEQ, their main() renamed away) into oracle/_ref/.  The loop
 * nest below restates the reference driver (gppComplex_seq.cpp:335-383,
 * gppKerSeq.cpp:266-314) with two generalisations the seeded workloads need:
 * wx may differ per band (wx_array[n1*wx_stride + iw]) and nw is a runtime
 * value.  Every arithmetic step of a term is done by the reference's own
 * flagOCC_solver / noflagOCC_solver / reduce_achstemp, so the outputs are the
 * reference's answers on the given inputs.  tests/golden/make_golden.py uses
 * them to pin the C restatement in gpp_oracle.c.
 */
#include "gpp_oracle.h"

#include <cstring>
#include <vector>

#if defined(REF_COMPLEX_SEQ)
#include "Complex.h"
typedef GPPComplex RC;
static inline RC rc(double re, double im) { return GPPComplex(re, im); }
static inline RC rc_scale(const RC &a, double s) { return GPPComplex_mult(a, s); }
static inline double rc_re(const RC &a) { return GPPComplex_real(a); }
static inline double rc_im(const RC &a) { return GPPComplex_imag(a); }
#elif defined(REF_KERSEQ)
#include <complex>
typedef std::complex<double> RC;
static inline RC rc(double re, double im) { return RC(re, im); }
static inline RC rc_scale(const RC &a, double s) { return a * s; }
static inline double rc_re(const RC &a) { return a.real(); }
static inline double rc_im(const RC &a) { return a.imag(); }
#else
#error "define REF_COMPLEX_SEQ or REF_KERSEQ"
#endif

/* The reference's functions, with their reference signatures
 * (gppComplex_seq.cpp:66,107,131 / gppKerSeq.cpp:67,106,127). */
void reduce_achstemp(int n1, int *inv_igp_index, int ncouls, RC *aqsmtemp, RC *aqsntemp,
                     RC *I_eps_array, RC &achstemp, int ngpown, double *vcoul);
void flagOCC_solver(double wxt, RC *wtilde_array, int my_igp, int n1, RC *aqsmtemp, RC *aqsntemp,
                    RC *I_eps_array, RC &ssxt, RC &scht, int ncouls, int igp, RC *ssxa, RC *scha);
void noflagOCC_solver(double wxt, RC *wtilde_array, int my_igp, int n1, RC *aqsmtemp, RC *aqsntemp,
                      RC *I_eps_array, RC &ssxt, RC &scht, int ncouls, int igp, RC *scha);

extern "C" int ref_sigma(const oracle_problem *p, oracle_outputs *o)
{
    if (!p || !o || !o->achtemp || !o->asxtemp || p->ncouls <= 0 || p->nw <= 0) return -1;
    const int nc = p->ncouls, ng = p->ngpown, nw = p->nw;
    if (o->acht_n1_loc && nw < 3) return -1;
    for (int i = 0; i < ng; ++i)
        if (p->inv_igp_index[i] < 0) return -1;

    RC *aqsm = reinterpret_cast<RC *>(const_cast<oracle_complex *>(p->aqsmtemp));
    RC *aqsn = reinterpret_cast<RC *>(const_cast<oracle_complex *>(p->aqsntemp));
    RC *ieps = reinterpret_cast<RC *>(const_cast<oracle_complex *>(p->I_eps_array));
    RC *wt = reinterpret_cast<RC *>(const_cast<oracle_complex *>(p->wtilde_array));
    int *inv = const_cast<int *>(p->inv_igp_index);
    double *vcoul = const_cast<double *>(p->vcoul);

    std::vector<RC> achtemp(nw, rc(0, 0)), asxtemp(nw, rc(0, 0)), ssx_array(nw, rc(0, 0)),
        sch_array(nw, rc(0, 0)), acht_n1(p->number_bands, rc(0, 0));
    std::vector<RC> ssxa(nc, rc(0, 0)), scha(nc, rc(0, 0));
    RC achstemp = rc(0, 0);

    for (int n1 = p->band_begin; n1 < p->band_end; ++n1) {
        const bool flag_occ = n1 < p->nvband;
        reduce_achstemp(n1, inv, nc, aqsm, aqsn, ieps, achstemp, ng, vcoul);
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            int igp = inv[my_igp];
            if (igp >= nc) igp = nc - 1;
            for (int i = 0; i < nw; ++i) { ssx_array[i] = rc(0, 0); sch_array[i] = rc(0, 0); }
            for (int iw = 0; iw < nw; ++iw) {
                RC scht = rc(0, 0), ssxt = rc(0, 0);
                const double wxt = p->wx_array[(size_t)n1 * p->wx_stride + iw];
                if (flag_occ) {
                    flagOCC_solver(wxt, wt, my_igp, n1, aqsm, aqsn, ieps, ssxt, scht, nc, igp,
                                   ssxa.data(), scha.data());
                    ssx_array[iw] += ssxt;
                    sch_array[iw] += rc_scale(scht, 0.5);
#if defined(REF_KERSEQ)
                    asxtemp[iw] += ssx_array[iw] * p->occ * vcoul[igp];
#else
                    asxtemp[iw] += rc_scale(ssx_array[iw], p->occ * vcoul[igp]);
#endif
                } else {
                    noflagOCC_solver(wxt, wt, my_igp, n1, aqsm, aqsn, ieps, ssxt, scht, nc, igp,
                                     scha.data());
                    sch_array[iw] += rc_scale(scht, 0.5);
                }
            }
            for (int iw = 0; iw < nw; ++iw) achtemp[iw] += rc_scale(sch_array[iw], vcoul[igp]);
            if (nw >= 3) acht_n1[n1] += rc_scale(sch_array[2], vcoul[igp]);
        }
    }
    for (int iw = 0; iw < nw; ++iw) {
        o->achtemp[iw].re = rc_re(achtemp[iw]); o->achtemp[iw].im = rc_im(achtemp[iw]);
        o->asxtemp[iw].re = rc_re(asxtemp[iw]); o->asxtemp[iw].im = rc_im(asxtemp[iw]);
    }
    if (o->acht_n1_loc)
        for (int n1 = 0; n1 < p->number_bands; ++n1) {
            o->acht_n1_loc[n1].re = rc_re(acht_n1[n1]); o->acht_n1_loc[n1].im = rc_im(acht_n1[n1]);
        }
    if (o->achstemp) { o->achstemp[0].re = rc_re(achstemp); o->achstemp[0].im = rc_im(achstemp); }
    return 0;
}

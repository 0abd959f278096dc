// gpp_compat.cpp -- the reference's own C++ entry points, re-exported with
// their exact signatures (and so their exact mangled symbol names) on top of
// the C ABI.  A host program written against the reference's GPPComplex.h
// (e.g. the unmodified gppCudaVer.cpp driver) links against libgpp_gb300.so
// in place of the reference's GPPComplex.o and runs the GB300 kernels.
//
// GPPComplex is only forward-declared: every argument is a pointer to the
// reference's 16-byte {double x, y} class (GPPComplex.h:68, a double2), which
// has the layout of gpp_complex.  Like the reference launchers
// (GPPComplex.cu:414-416, 430-432) these functions return nothing and print
// the error on failure; the C entry points report it as a status instead.
#include <cstdio>

#include "gpp_gb300.h"

class GPPComplex;

namespace {
inline const gpp_complex *cc(const GPPComplex *p) { return reinterpret_cast<const gpp_complex *>(p); }
inline gpp_complex *mc(GPPComplex *p) { return reinterpret_cast<gpp_complex *>(p); }
inline void report(gpp_status st) {
    if (st != GPP_OK) printf("Error: %s\n", gpp_last_error_message());
}
}  // namespace

// GPPComplex.h:304 (declared there, never defined in the reference).
void gppKernelGPU(GPPComplex *wtilde_array, GPPComplex *aqsntemp, GPPComplex *aqsmtemp,
                  GPPComplex *I_eps_array, int ncouls, int ngpown, int number_bands,
                  double *wx_array, double *achtemp_re, double *achtemp_im, double *vcoul,
                  int nstart, int nend, int *indinv, int *inv_igp_index) {
    report(gpp_kernel_gpu(cc(wtilde_array), cc(aqsntemp), cc(aqsmtemp), cc(I_eps_array), ncouls,
                          ngpown, number_bands, wx_array, achtemp_re, achtemp_im, vcoul, nstart,
                          nend, indinv, inv_igp_index));
}

// GPPComplex.cu:406 / GPPComplex.h:306.
void d_till_nvband(int nvband, int ngpown, int ncouls, int *inv_igp_index, double *wx_array,
                   GPPComplex *wtilde_array, GPPComplex *aqsmtemp, GPPComplex *aqsntemp,
                   GPPComplex *I_eps_array, GPPComplex *asxtemp, double *vcoul,
                   GPPComplex *acht_n1_loc, double *achtemp_re, double *achtemp_im,
                   const double occ) {
    report(gpp_till_nvband(nvband, ngpown, ncouls, inv_igp_index, wx_array, cc(wtilde_array),
                           cc(aqsmtemp), cc(aqsntemp), cc(I_eps_array), mc(asxtemp), vcoul,
                           mc(acht_n1_loc), achtemp_re, achtemp_im, occ));
}

// GPPComplex.cu:422 / GPPComplex.h:310.
void d_noFlagOCCSolver(int number_bands, int nvband, int ngpown, int ncouls, int *inv_igp_index,
                       double *wx_array, GPPComplex *wtilde_array, GPPComplex *aqsmtemp,
                       GPPComplex *aqsntemp, GPPComplex *I_eps_array, double *vcoul,
                       double *achtemp_re, double *achtemp_im, GPPComplex *acht_n1_loc) {
    report(gpp_noflag_occ_solver(number_bands, nvband, ngpown, ncouls, inv_igp_index, wx_array,
                                 cc(wtilde_array), cc(aqsmtemp), cc(aqsntemp), cc(I_eps_array),
                                 vcoul, achtemp_re, achtemp_im, mc(acht_n1_loc)));
}

// GPPComplex.h:308 (declared there, never defined in the reference): the
// static term into split real/imaginary accumulators.
extern "C" gpp_status gpp_reduce_achstemp_split(int number_bands, const int *inv_igp_index,
                                                int ncouls, const gpp_complex *aqsmtemp,
                                                const gpp_complex *aqsntemp,
                                                const gpp_complex *I_eps_array, double *re,
                                                double *im, int ngpown, const double *vcoul);

void d_reduce_achstemp(int number_bands, int *inv_igp_index, int ncouls, GPPComplex *aqsmtemp,
                       GPPComplex *aqsntemp, GPPComplex *I_eps_array, double *achstemp_re,
                       double *achstemp_im, int ngpown, double *vcoul) {
    report(gpp_reduce_achstemp_split(number_bands, inv_igp_index, ncouls, cc(aqsmtemp),
                                     cc(aqsntemp), cc(I_eps_array), achstemp_re, achstemp_im,
                                     ngpown, vcoul));
}

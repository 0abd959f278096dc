// gpp_driver.cpp -- host program that drives the GB300 kernels exactly the
// way the reference's CUDA driver does (gppCudaVer.cpp:236-425): synthesise
// the ramp inputs, copy them to the device, call the reference's entry points
// d_till_nvband and d_noFlagOCCSolver (re-exported by libgpp_gb300.so with
// the reference's signatures), synchronise and print achtemp.
//
//   gpp_driver.ex <number_bands> <nvband> <ncouls> <nodes_per_group>
//
// Output lines "achtemp[iw] = (re,im)" use 15 significant digits, the format
// of gppKerSeq.cpp:321-322, so the README known answers can be compared
// directly.  Exit status is non-zero on any CUDA or library error.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gpp_gb300.h"

class GPPComplex;  // the reference's 16-byte complex (GPPComplex.h:68)

// The reference's entry points (GPPComplex.h:306,310), provided by libgpp_gb300.so.
void d_till_nvband(int nvband, int ngpown, int ncouls, int *inv_igp_index, double *wx_array,
                   GPPComplex *wtilde_array, GPPComplex *aqsmtemp, GPPComplex *aqsntemp,
                   GPPComplex *I_eps_array, GPPComplex *asxtemp, double *vcoul,
                   GPPComplex *acht_n1_loc, double *achtemp_re, double *achtemp_im,
                   const double occ);
void d_noFlagOCCSolver(int number_bands, int nvband, int ngpown, int ncouls, int *inv_igp_index,
                       double *wx_array, GPPComplex *wtilde_array, GPPComplex *aqsmtemp,
                       GPPComplex *aqsntemp, GPPComplex *I_eps_array, double *vcoul,
                       double *achtemp_re, double *achtemp_im, GPPComplex *acht_n1_loc);

#define CHECK(call)                                                                 \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return 2;                                                               \
        }                                                                           \
    } while (0)

int main(int argc, char **argv) {
    if (argc != 5) {
        printf("usage: %s <number_bands> <nvband> <ncouls> <nodes_per_group>\n", argv[0]);
        return 1;
    }
    const int nb = atoi(argv[1]), nv = atoi(argv[2]), nc = atoi(argv[3]), npg = atoi(argv[4]);
    if (nb <= 0 || nv < 0 || nv > nb || nc <= 0 || npg <= 0 || nc / npg <= 0) {
        fprintf(stderr, "invalid sizes\n");
        return 1;
    }
    const int ng = nc / npg;
    const int nw = 3;
    // Ramp inputs of the mini-app: (i+j)(0.5+0.5i), vcoul[i] = i,
    // inv_igp_index[i] = (i+1) ncouls / ngpown, wx = e_lk - e_n1kq + dw (iw-1).
    std::vector<gpp_complex> aqs((size_t)nb * nc), gmat((size_t)ng * nc);
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nc; ++j) aqs[(size_t)i * nc + j] = {0.5 * (i + j), 0.5 * (i + j)};
    for (int i = 0; i < ng; ++i)
        for (int j = 0; j < nc; ++j) gmat[(size_t)i * nc + j] = {0.5 * (i + j), 0.5 * (i + j)};
    std::vector<int> inv(ng);
    for (int i = 0; i < ng; ++i) inv[i] = (int)((long long)(i + 1) * nc / ng);
    std::vector<double> vcoul(nc);
    for (int i = 0; i < nc; ++i) vcoul[i] = 1.0 * i;
    double wx[nw];
    for (int iw = 0; iw < nw; ++iw) {
        wx[iw] = 10.0 - 6.0 + 1.0 * ((iw + 1) - 2);
        if (std::fabs(wx[iw]) < 1e-6) wx[iw] = 1e-6;
    }

    gpp_complex *d_aqsm, *d_aqsn, *d_ieps, *d_wt, *d_asx, *d_n1;
    double *d_vcoul, *d_wx, *d_re, *d_im;
    int *d_inv;
    CHECK(cudaMalloc(&d_aqsm, aqs.size() * 16));
    CHECK(cudaMalloc(&d_aqsn, aqs.size() * 16));
    CHECK(cudaMalloc(&d_ieps, gmat.size() * 16));
    CHECK(cudaMalloc(&d_wt, gmat.size() * 16));
    CHECK(cudaMalloc(&d_asx, nw * 16));
    CHECK(cudaMalloc(&d_n1, (size_t)nb * 16));
    CHECK(cudaMalloc(&d_vcoul, nc * 8));
    CHECK(cudaMalloc(&d_wx, nw * 8));
    CHECK(cudaMalloc(&d_re, nw * 8));
    CHECK(cudaMalloc(&d_im, nw * 8));
    CHECK(cudaMalloc(&d_inv, ng * 4));
    CHECK(cudaMemcpy(d_aqsm, aqs.data(), aqs.size() * 16, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_aqsn, aqs.data(), aqs.size() * 16, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_ieps, gmat.data(), gmat.size() * 16, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_wt, gmat.data(), gmat.size() * 16, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_vcoul, vcoul.data(), nc * 8, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_wx, wx, nw * 8, cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_inv, inv.data(), ng * 4, cudaMemcpyHostToDevice));
    CHECK(cudaMemset(d_re, 0, nw * 8));
    CHECK(cudaMemset(d_im, 0, nw * 8));
    CHECK(cudaMemset(d_asx, 0, nw * 16));
    CHECK(cudaMemset(d_n1, 0, (size_t)nb * 16));

    auto t0 = std::chrono::steady_clock::now();
    GPPComplex *wt = reinterpret_cast<GPPComplex *>(d_wt);
    GPPComplex *am = reinterpret_cast<GPPComplex *>(d_aqsm);
    GPPComplex *an = reinterpret_cast<GPPComplex *>(d_aqsn);
    GPPComplex *ie = reinterpret_cast<GPPComplex *>(d_ieps);
    d_till_nvband(nv, ng, nc, d_inv, d_wx, wt, am, an, ie, reinterpret_cast<GPPComplex *>(d_asx),
                  d_vcoul, reinterpret_cast<GPPComplex *>(d_n1), d_re, d_im, 1.0);
    d_noFlagOCCSolver(nb, nv, ng, nc, d_inv, d_wx, wt, am, an, ie, d_vcoul, d_re, d_im,
                      reinterpret_cast<GPPComplex *>(d_n1));
    CHECK(cudaDeviceSynchronize());
    const gpp_status st = gpp_wait(nullptr, -1);
    if (st != GPP_OK) {
        fprintf(stderr, "gpp error: %s\n", gpp_last_error_message());
        return 3;
    }
    double re[nw], im[nw];
    CHECK(cudaMemcpy(re, d_re, nw * 8, cudaMemcpyDeviceToHost));
    CHECK(cudaMemcpy(im, d_im, nw * 8, cudaMemcpyDeviceToHost));
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int iw = 0; iw < nw; ++iw) printf("achtemp[%d] = (%.15g,%.15g)\n", iw, re[iw], im[iw]);
    printf("********** Time Taken **********= %g secs\n", secs);
    cudaFree(d_aqsm); cudaFree(d_aqsn); cudaFree(d_ieps); cudaFree(d_wt); cudaFree(d_asx);
    cudaFree(d_n1); cudaFree(d_vcoul); cudaFree(d_wx); cudaFree(d_re); cudaFree(d_im);
    cudaFree(d_inv);
    return 0;
}

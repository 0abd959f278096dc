"""The coarse/fine form of Re(wtilde) and wx (coarse_fine, gpp_df.cuh) and the
fused float-float reciprocal product (df2_mul_rcp, gpp_df2.cuh) of the mixed
kernels, checked with the same code compiled for the host here (and for the
device on a GPU):

* the coarse part lies on the 2^-18 grid, |c| <= 16, and c + f equals the
  FP64 value to within 2^-43 + 2^-45;
* coarse parts of any two such values subtract exactly in FP32, which is
  what lets the kernel form Re(wdiff) = wx - Re(wtilde) with one subtraction;
* values with |x| >= 16, Inf or NaN are left in (hi, lo) form and reported;
* a / d through df2_rcp_parts + df2_mul_rcp is within 2^-42 of the exact
  quotient (the float-float error budget of a term), without a sign
  preference over many terms.
"""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

CSRC = os.path.join(REPO, "doe-csfg-hackathon_gb300", "csrc")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include "gpp_df2.cuh"

using gpp::df;
using gpp::df2;

static unsigned long long next(unsigned long long &s) {  // SplitMix64
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double unit(unsigned long long &s) { return (next(s) >> 11) * (1.0 / 9007199254740992.0); }

// coarse_fine on both sides of the check (host or device), results compared
// in FP64 on the host.
struct CF { df v; int ok; };

#ifdef ON_DEVICE
__global__ void cf_kernel(const double *x, CF *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        df v = gpp::split(x[i]);
        const bool ok = gpp::coarse_fine(v);
        out[i] = CF{v, ok ? 1 : 0};
    }
}
__global__ void sub_kernel(const CF *a, const CF *b, float *d, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = __fsub_rn(a[i].v.h, b[i].v.h);
}
#endif

int main() {
    unsigned long long s = 2024;
    std::vector<double> x;
    for (int i = 0; i < 1000000; ++i) x.push_back(-16.0 + 32.0 * unit(s));       // whole range
    for (int i = 0; i < 200000; ++i) x.push_back((unit(s) - 0.5) * 1e-3);        // tiny
    for (int i = 0; i < 200000; ++i) x.push_back(0.5 + 1.5 * unit(s));           // wtilde-like
    for (int i = 0; i < 100000; ++i) x.push_back(ldexp(std::floor((unit(s) - 0.5) * 8e6), -18));  // on the grid, |x| < 16
    for (double v : {0.0, -0.0, 16.0 - ldexp(1.0, -20), -16.0 + ldexp(1.0, -20),
                     1e-300, ldexp(1.0, -19), ldexp(3.0, -20)})
        x.push_back(v);
    const size_t n_in = x.size();
    // Out of range: |hi| >= 16 (15.999999999 rounds to the float 16), Inf, NaN.
    for (double v : {16.0, -16.0, 15.999999999, -15.999999999, 17.5, 1e6, (double)INFINITY,
                     -(double)INFINITY, (double)NAN})
        x.push_back(v);
    const int n = (int)x.size();
    std::vector<CF> cf(n);
#ifdef ON_DEVICE
    double *dx; CF *dcf;
    if (cudaMalloc(&dx, 8 * n) || cudaMalloc(&dcf, sizeof(CF) * n)) return 3;
    cudaMemcpy(dx, x.data(), 8 * n, cudaMemcpyHostToDevice);
    cf_kernel<<<(n + 255) / 256, 256>>>(dx, dcf, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    cudaMemcpy(cf.data(), dcf, sizeof(CF) * n, cudaMemcpyDeviceToHost);
#else
    for (int i = 0; i < n; ++i) {
        df v = gpp::split(x[i]);
        const bool ok = gpp::coarse_fine(v);
        cf[i] = CF{v, ok ? 1 : 0};
    }
#endif
    int bad = 0;
    double worst = 0.0;
    for (int i = 0; i < n; ++i) {
        const bool in_range = (size_t)i < n_in;
        if (cf[i].ok != (in_range ? 1 : 0)) { if (bad++ < 5) printf("range flag x=%a\n", x[i]); continue; }
        if (!in_range) {
            df w = gpp::split(x[i]);
            if (memcmp(&w, &cf[i].v, sizeof(df)) != 0 && x[i] == x[i]) {
                if (bad++ < 5) printf("out-of-range value changed x=%a\n", x[i]);
            }
            continue;
        }
        const double c = cf[i].v.h, f = cf[i].v.l;
        const double k = ldexp(c, 18);
        // |f| <= 2^-19 (half the grid) + |lo| (<= 2^-21 below 16).
        if (k != std::floor(k) || std::fabs(c) > 16.0 || std::fabs(f) > ldexp(5.0, -21)) {
            if (bad++ < 5) printf("coarse part off the grid x=%a c=%a f=%a\n", x[i], c, f);
        }
        const double err = std::fabs((c + f) - x[i]);
        if (err > worst) worst = err;
        // One rounding of f (2^-43) plus that of the float-float split (2^-45).
        if (err > ldexp(5.0, -45)) { if (bad++ < 5) printf("c+f off x=%a err=%g\n", x[i], err); }
    }
    // Exact subtraction of the coarse parts of random pairs.
    std::vector<CF> a(n_in), b(n_in);
    for (size_t i = 0; i < n_in; ++i) { a[i] = cf[i]; b[i] = cf[(i * 7919 + 13) % n_in]; }
    std::vector<float> d(n_in);
#ifdef ON_DEVICE
    CF *da, *db; float *dd;
    if (cudaMalloc(&da, sizeof(CF) * n_in) || cudaMalloc(&db, sizeof(CF) * n_in) ||
        cudaMalloc(&dd, 4 * n_in)) return 3;
    cudaMemcpy(da, a.data(), sizeof(CF) * n_in, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b.data(), sizeof(CF) * n_in, cudaMemcpyHostToDevice);
    sub_kernel<<<((int)n_in + 255) / 256, 256>>>(da, db, dd, (int)n_in);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    cudaMemcpy(d.data(), dd, 4 * n_in, cudaMemcpyDeviceToHost);
#else
    for (size_t i = 0; i < n_in; ++i) d[i] = gpp::fsub(a[i].v.h, b[i].v.h);
#endif
    for (size_t i = 0; i < n_in; ++i) {
        const double exact = (double)a[i].v.h - (double)b[i].v.h;
        if ((double)d[i] != exact) { if (bad++ < 5) printf("inexact coarse difference %a - %a\n", a[i].v.h, b[i].v.h); }
    }
    // Fused reciprocal products: a / d for df a and positive df d.
    double max_rel = 0.0, mean_signed = 0.0;
    const int m = 400000;
    for (int i = 0; i < m; ++i) {
        const double av = (unit(s) - 0.5) * 8.0, dv = ldexp(0.25 + unit(s), (int)(next(s) % 40) - 20);
        const df ah = gpp::split(av), dh = gpp::split(dv);
        const df2 A = gpp::df2_bcast(ah), D = gpp::df2_bcast(dh);
        float2 r0, rc;
        gpp::df2_rcp_parts(D, r0, rc);
        const df2 q = gpp::df2_mul_rcp(A, r0, rc);
        const long double want = ((long double)ah.h + ah.l) / ((long double)dh.h + dh.l);
        const long double got = (long double)q.h.x + q.l.x;
        if (want != 0) {
            const double rel = (double)((got - want) / want);
            mean_signed += rel;
            if (std::fabs(rel) > max_rel) max_rel = std::fabs(rel);
        }
    }
    mean_signed /= m;
    printf("coarse/fine worst |c+f-x| = %g; quotient max rel %g, mean signed %g\n", worst, max_rel,
           mean_signed);
    if (max_rel > ldexp(1.0, -42)) { printf("quotient error too large\n"); ++bad; }
    if (std::fabs(mean_signed) > ldexp(1.0, -50)) { printf("quotient error biased\n"); ++bad; }
    printf("%d failures\n", bad);
    return bad ? 1 : 0;
}
"""


def _run(tmp_path, device):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = tmp_path / "coarse_fine_check.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "coarse_fine_check"
    # Device code for sm_103a even for the host run: the packed f32x2
    # intrinsics the header's device branch uses exist from sm_100 on.
    cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-gencode",
           "arch=compute_103a,code=sm_103a", "-I", CSRC, str(src), "-o", str(exe)]
    if device:
        cmd += ["-DON_DEVICE"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 failures" in out.stdout


def test_coarse_fine_and_fused_reciprocal_on_the_host(tmp_path):
    _run(tmp_path, device=False)


@pytest.mark.gpu
def test_coarse_fine_on_the_device(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _run(tmp_path, device=True)

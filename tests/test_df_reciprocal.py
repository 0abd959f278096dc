"""The fused float-float reciprocal product of the mixed kernels
(df2_rcp_parts + df2_mul_rcp, gpp_df2.cuh): a / d with the second-order
Newton correction of the reciprocal folded into the product, checked with
the same code compiled for the host here (and for the device on a GPU).  It
must stay within 2^-42 of the exact quotient (the float-float error budget
of a term) and carry no sign preference over many terms.
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

#ifdef ON_DEVICE
__global__ void quot_kernel(const df *a, const df *d, df *q, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float2 r0, rc;
        gpp::df2_rcp_parts(gpp::df2_bcast(d[i]), r0, rc);
        const df2 v = gpp::df2_mul_rcp(gpp::df2_bcast(a[i]), r0, rc);
        q[i] = df{v.h.x, v.l.x};
    }
}
#endif

int main() {
    unsigned long long s = 2024;
    const int m = 400000;
    std::vector<df> a(m), d(m), q(m);
    for (int i = 0; i < m; ++i) {
        a[i] = gpp::split((unit(s) - 0.5) * 8.0);
        d[i] = gpp::split(ldexp(0.25 + unit(s), (int)(next(s) % 40) - 20));
    }
#ifdef ON_DEVICE
    df *da, *dd, *dq;
    if (cudaMalloc(&da, 8 * m) || cudaMalloc(&dd, 8 * m) || cudaMalloc(&dq, 8 * m)) return 3;
    cudaMemcpy(da, a.data(), 8 * m, cudaMemcpyHostToDevice);
    cudaMemcpy(dd, d.data(), 8 * m, cudaMemcpyHostToDevice);
    quot_kernel<<<(m + 255) / 256, 256>>>(da, dd, dq, m);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    cudaMemcpy(q.data(), dq, 8 * m, cudaMemcpyDeviceToHost);
#else
    for (int i = 0; i < m; ++i) {
        float2 r0, rc;
        gpp::df2_rcp_parts(gpp::df2_bcast(d[i]), r0, rc);
        const df2 v = gpp::df2_mul_rcp(gpp::df2_bcast(a[i]), r0, rc);
        q[i] = df{v.h.x, v.l.x};
    }
#endif
    double max_rel = 0.0, mean_signed = 0.0;
    for (int i = 0; i < m; ++i) {
        const long double want = ((long double)a[i].h + a[i].l) / ((long double)d[i].h + d[i].l);
        const long double got = (long double)q[i].h + q[i].l;
        if (want != 0) {
            const double rel = (double)((got - want) / want);
            mean_signed += rel;
            if (std::fabs(rel) > max_rel) max_rel = std::fabs(rel);
        }
    }
    mean_signed /= m;
    printf("quotient max rel %g, mean signed %g\n", max_rel, mean_signed);
    int bad = 0;
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
    src = tmp_path / "reciprocal_check.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "reciprocal_check"
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


def test_fused_reciprocal_product_on_the_host(tmp_path):
    _run(tmp_path, device=False)


@pytest.mark.gpu
def test_fused_reciprocal_product_on_the_device(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _run(tmp_path, device=True)

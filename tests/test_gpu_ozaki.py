"""The FP64-accurate tensor-core GEMM (gpp_ozaki.cu, tcgen05) on its own:
a harness linked against libgpp_gb300.so calls gpp::ozaki_zgemm on complex
operands in both layouts (k contiguous or rows contiguous), with ragged
sizes, several k chunks and k splits, a wide dynamic range along k, and
operands whose slices take the extreme values (s_1 = 128, s_2..s_8 = -64:
the group sums reach 2^23, where FP32 accumulation must still be exact), and
compares with sums in long double; an Inf or NaN input turns its row's or
column's results into NaN and leaves the others alone; small integer operands
give the exact integer result, bit for bit.  The bound is 1e-13 of the largest
result, normwise (an FP64 3M-form GEMM is ~1e-15 to 1e-14 here); the
device fault word must stay clear.
"""
import os
import shutil
import subprocess

import pytest

from conftest import REPO
from gppsigma import build

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CSRC = os.path.join(REPO, "doe-csfg-hackathon_gb300", "csrc")
INCLUDE = os.path.join(REPO, "include")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <vector>
#include <cuda_runtime.h>
#include "gpp_ozaki.h"

static unsigned long long st = 99;
static double uni() {
    unsigned long long z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (z >> 11) * (1.0 / 9007199254740992.0);
}

// 2^e sum_i s_i 128^-i with s = (128, -64, ..., -64): the largest slices.
static double extreme() {
    double v = 1.0;
    for (int i = 2; i <= 8; ++i) v -= 64.0 * std::ldexp(1.0, -7 * i);
    return v;
}

static int run(int M, int N, int K, int splits, bool kfast, double range, bool ext) {
    std::vector<double2> X((size_t)M * K), Y((size_t)N * K);
    const double xe = extreme();
    for (auto &v : X) {
        const double s = std::exp((uni() - 0.5) * range);
        v = ext ? make_double2(xe, -xe) : make_double2((uni() - 0.5) * s, (uni() - 0.5) * s);
    }
    // (x, -x): the re + im plane is zero, so re and im keep the common exponent 0 and
    // their extreme slices.
    for (auto &v : Y) v = ext ? make_double2(xe, -xe) : make_double2(uni() - 0.5, uni() - 0.5);
    std::vector<double2> Xd(X.size()), Yd(Y.size());
    for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k)
            Xd[kfast ? (size_t)m * K + k : (size_t)k * M + m] = X[(size_t)m * K + k];
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < K; ++k)
            Yd[kfast ? (size_t)n * K + k : (size_t)k * N + n] = Y[(size_t)n * K + k];
    const int zs = gpp::ozaki_splits(K, splits);
    double2 *dX, *dY, *dO;
    void *ws;
    int *derr;
    if (cudaMalloc(&dX, X.size() * 16) || cudaMalloc(&dY, Y.size() * 16) ||
        cudaMalloc(&dO, (size_t)zs * M * N * 16) ||
        cudaMalloc(&ws, gpp::ozaki_bytes(M, N, K, splits)) || cudaMalloc(&derr, 4))
        return 3;
    cudaMemcpy(dX, Xd.data(), X.size() * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(dY, Yd.data(), Y.size() * 16, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, 4);
    const gpp::OzOperand ox{dX, kfast ? K : M, kfast, M}, oy{dY, kfast ? K : N, kfast, N};
    if (gpp::ozaki_zgemm(ox, oy, M, N, K, splits, dO, N, (long long)M * N, ws, derr, 0) !=
            cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
        return 4;
    int herr = 0;
    cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
    std::vector<double2> O((size_t)zs * M * N);
    cudaMemcpy(O.data(), dO, O.size() * 16, cudaMemcpyDeviceToHost);
    double maxerr = 0, maxref = 0;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            long double re = 0, im = 0;
            for (int k = 0; k < K; ++k) {
                const double2 a = X[(size_t)m * K + k], b = Y[(size_t)n * K + k];
                re += (long double)a.x * b.x - (long double)a.y * b.y;
                im += (long double)a.x * b.y + (long double)a.y * b.x;
            }
            double gre = 0, gim = 0;
            for (int z = 0; z < zs; ++z) {
                gre += O[((size_t)z * M + m) * N + n].x;
                gim += O[((size_t)z * M + m) * N + n].y;
            }
            maxerr = std::fmax(maxerr, std::fmax(std::fabs(gre - (double)re), std::fabs(gim - (double)im)));
            maxref = std::fmax(maxref, std::fmax(std::fabs((double)re), std::fabs((double)im)));
        }
    const double rel = maxerr / maxref;
    unsigned long long hash = 1469598103934665603ull;  // FNV-1a over the result's bits
    const unsigned char *bytes = reinterpret_cast<const unsigned char *>(O.data());
    for (size_t i = 0; i < O.size() * sizeof(double2); ++i) hash = (hash ^ bytes[i]) * 1099511628211ull;
    printf("M %d N %d K %d splits %d kfast %d range %g extreme %d: normwise %.3e, fault word %d, "
           "bits %016llx\n",
           M, N, K, zs, (int)kfast, range, (int)ext, rel, herr, hash);
    cudaFree(dX); cudaFree(dY); cudaFree(dO); cudaFree(ws); cudaFree(derr);
    return (rel <= 1e-13 && herr == 0) ? 0 : 1;
}

// An Inf in row 3 of X and a NaN in row 5 of Y: the results of that row and
// that column are NaN, every other result as without them.
static int run_nonfinite() {
    const int M = 40, N = 70, K = 600;
    std::vector<double2> X((size_t)K * M), Y((size_t)K * N);
    for (auto &v : X) v = make_double2(uni() - 0.5, uni() - 0.5);
    for (auto &v : Y) v = make_double2(uni() - 0.5, uni() - 0.5);
    std::vector<double2> Xc = X, Yc = Y;  // k-major: X[k * M + m]
    X[(size_t)550 * M + 3].x = INFINITY;
    Y[(size_t)7 * N + 5].y = NAN;
    const int zs = gpp::ozaki_splits(K, 1);
    double2 *dX, *dY, *dO, *dOc;
    void *ws;
    int *derr;
    if (cudaMalloc(&dX, X.size() * 16) || cudaMalloc(&dY, Y.size() * 16) ||
        cudaMalloc(&dO, (size_t)zs * M * N * 16) || cudaMalloc(&dOc, (size_t)zs * M * N * 16) ||
        cudaMalloc(&ws, gpp::ozaki_bytes(M, N, K, 1)) || cudaMalloc(&derr, 4))
        return 3;
    cudaMemset(derr, 0, 4);
    const gpp::OzOperand ox{dX, M, false, M}, oy{dY, N, false, N};
    cudaMemcpy(dX, X.data(), X.size() * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(dY, Y.data(), Y.size() * 16, cudaMemcpyHostToDevice);
    gpp::ozaki_zgemm(ox, oy, M, N, K, 1, dO, N, (long long)M * N, ws, derr, 0);
    cudaMemcpy(dX, Xc.data(), X.size() * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(dY, Yc.data(), Y.size() * 16, cudaMemcpyHostToDevice);
    gpp::ozaki_zgemm(ox, oy, M, N, K, 1, dOc, N, (long long)M * N, ws, derr, 0);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    std::vector<double2> O((size_t)M * N), Oc((size_t)M * N);
    cudaMemcpy(O.data(), dO, O.size() * 16, cudaMemcpyDeviceToHost);
    cudaMemcpy(Oc.data(), dOc, Oc.size() * 16, cudaMemcpyDeviceToHost);
    int bad = 0;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            const double2 o = O[(size_t)m * N + n], c = Oc[(size_t)m * N + n];
            if (m == 3 || n == 5) {
                if (!(std::isnan(o.x) && std::isnan(o.y))) ++bad;
            } else if (std::fabs(o.x - c.x) > 1e-12 * std::fabs(c.x) + 1e-300 ||
                       std::fabs(o.y - c.y) > 1e-12 * std::fabs(c.y) + 1e-300) {
                ++bad;
            }
        }
    printf("non-finite inputs: %d wrong results\n", bad);
    cudaFree(dX); cudaFree(dY); cudaFree(dO); cudaFree(dOc); cudaFree(ws); cudaFree(derr);
    return bad ? 1 : 0;
}

// Integer operands, |re|, |im| <= 2^(bits - 1): every slice product, group
// sum, packed pair and float-float sum is exact, and so is the 3M
// combination of integers, so the GEMM must equal the exact integer result
// bit for bit.
static int run_exact(int M, int N, int K, bool kfast, int bits) {
    std::vector<double2> X((size_t)M * K), Y((size_t)N * K);
    const long long span = 1ll << bits;
    auto rnd = [&]() { return (double)((long long)(uni() * span) - span / 2); };
    for (auto &v : X) v = make_double2(rnd(), rnd());
    for (auto &v : Y) v = make_double2(rnd(), rnd());
    std::vector<double2> Xd(X.size()), Yd(Y.size());
    for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k)
            Xd[kfast ? (size_t)m * K + k : (size_t)k * M + m] = X[(size_t)m * K + k];
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < K; ++k)
            Yd[kfast ? (size_t)n * K + k : (size_t)k * N + n] = Y[(size_t)n * K + k];
    double2 *dX, *dY, *dO;
    void *ws;
    int *derr;
    if (cudaMalloc(&dX, X.size() * 16) || cudaMalloc(&dY, Y.size() * 16) ||
        cudaMalloc(&dO, (size_t)M * N * 16) || cudaMalloc(&ws, gpp::ozaki_bytes(M, N, K, 1)) ||
        cudaMalloc(&derr, 4))
        return 3;
    cudaMemcpy(dX, Xd.data(), X.size() * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(dY, Yd.data(), Y.size() * 16, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, 4);
    const gpp::OzOperand ox{dX, kfast ? K : M, kfast, M}, oy{dY, kfast ? K : N, kfast, N};
    if (gpp::ozaki_zgemm(ox, oy, M, N, K, 1, dO, N, 0, ws, derr, 0) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
        return 4;
    std::vector<double2> O((size_t)M * N);
    cudaMemcpy(O.data(), dO, O.size() * 16, cudaMemcpyDeviceToHost);
    long long wrong = 0;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            long long re = 0, im = 0;
            for (int k = 0; k < K; ++k) {
                const double2 a = X[(size_t)m * K + k], b = Y[(size_t)n * K + k];
                re += (long long)a.x * (long long)b.x - (long long)a.y * (long long)b.y;
                im += (long long)a.x * (long long)b.y + (long long)a.y * (long long)b.x;
            }
            const double2 o = O[(size_t)m * N + n];
            if (o.x != (double)re || o.y != (double)im) ++wrong;
        }
    printf("exact: M %d N %d K %d kfast %d, %d-bit integers: %lld results differ\n", M, N, K,
           (int)kfast, bits, wrong);
    cudaFree(dX); cudaFree(dY); cudaFree(dO); cudaFree(ws); cudaFree(derr);
    return wrong ? 1 : 0;
}

int main() {
    int bad = 0;
    bad |= run_exact(70, 300, 500, false, 15);
    bad |= run_exact(45, 260, 1700, true, 13);
    bad |= run_nonfinite();
    bad |= run(37, 300, 510, 1, false, 0, false);
    bad |= run(64, 128, 32, 1, false, 0, false);
    bad |= run(100, 257, 5, 1, true, 0, false);
    bad |= run(70, 200, 1500, 4, true, 0, false);
    bad |= run(50, 190, 2100, 3, false, 20, false);
    bad |= run(130, 300, 1024, 2, true, 0, true);
    bad |= run(129, 257, 512, 1, false, 0, true);
    printf("%s\n", bad ? "FAILED" : "all ok");
    return bad;
}
"""


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()


def test_tensor_core_fp64_gemm_against_long_double(tmp_path):
    """Also run in passes over single row tiles (a 1 MB budget for the stored
    group sums): the results must keep their bits."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    libdir = os.path.dirname(build.LIB)
    src = tmp_path / "ozaki_check.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "ozaki_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", CSRC, "-I", INCLUDE, str(src), "-o", str(exe), "-L", libdir,
                        "-lgpp_gb300", "-Xlinker", "-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "all ok" in out.stdout
    env = dict(os.environ, GPP_OZAKI_FOLD_MB="1")
    slabs = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600, env=env)
    assert slabs.returncode == 0, slabs.stdout + slabs.stderr
    assert slabs.stdout == out.stdout

"""split_bits (the integer-operation double -> float-float split of the prep
kernels) gives the same bits as split() (two FP64 conversions and an FP64
subtraction): on the host here, and on the device."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

CSRC = os.path.join(REPO, "doe-csfg-hackathon_gb300", "csrc")

HARNESS = r"""
#include <cstdio>
#include <cstring>
#include <vector>
#include "gpp_df.cuh"

using gpp::df;

static unsigned long long next(unsigned long long &s) {  // SplitMix64
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static std::vector<double> values() {
    std::vector<unsigned long long> bits;
    unsigned long long s = 12345;
    for (int i = 0; i < 2000000; ++i) {  // any exponent
        bits.push_back(next(s));
    }
    for (int i = 0; i < 2000000; ++i) {  // exponents around the fast range
        const unsigned long long e = 940 + next(s) % 150;
        bits.push_back((next(s) & 0x800fffffffffffffull) | (e << 52));
    }
    for (unsigned long long e : {0ull, 1ull, 962ull, 963ull, 1023ull, 1071ull, 1072ull, 2047ull})
        for (unsigned long long sign : {0ull, 1ull})
            for (unsigned long long m : {0ull, 1ull, 0x10000000ull, 0x30000000ull, 0x10000001ull,
                                         0xfffffffffffffull, 0xfffff0fffffffull,
                                         0xfffffe0000000ull | 0x10000000ull,
                                         0x0000020000000ull | 0x10000000ull})
                bits.push_back((sign << 63) | (e << 52) | m);
    std::vector<double> v(bits.size());
    memcpy(v.data(), bits.data(), 8 * bits.size());
    return v;
}

static bool same(df a, df b) { return memcmp(&a, &b, sizeof(df)) == 0; }

#ifdef ON_DEVICE
__global__ void both(const double *x, df *a, df *b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        a[i] = gpp::split_bits(x[i]);
        b[i] = gpp::split(x[i]);
    }
}
#endif

int main() {
    const std::vector<double> v = values();
    const int n = (int)v.size();
    std::vector<df> a(n), b(n);
#ifdef ON_DEVICE
    double *dx;
    df *da, *db;
    if (cudaMalloc(&dx, 8 * n) || cudaMalloc(&da, 8 * n) || cudaMalloc(&db, 8 * n)) return 3;
    cudaMemcpy(dx, v.data(), 8 * n, cudaMemcpyHostToDevice);
    both<<<(n + 255) / 256, 256>>>(dx, da, db, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    cudaMemcpy(a.data(), da, 8 * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), db, 8 * n, cudaMemcpyDeviceToHost);
#else
    for (int i = 0; i < n; ++i) {
        a[i] = gpp::split_bits(v[i]);
        b[i] = gpp::split(v[i]);
    }
#endif
    int bad = 0;
    for (int i = 0; i < n; ++i)
        if (!same(a[i], b[i]) && !(v[i] != v[i])) {  // NaN payloads aside
            if (bad < 5) printf("mismatch x=%a: (%a, %a) vs (%a, %a)\n", v[i], a[i].h, a[i].l, b[i].h, b[i].l);
            ++bad;
        }
    printf("checked %d values, %d mismatches\n", n, bad);
    return bad ? 1 : 0;
}
"""


def _run(tmp_path, device):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = tmp_path / "split_check.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "split_check"
    cmd = [nvcc, "-std=c++17", "-O2", "-I", CSRC, str(src), "-o", str(exe)]
    if device:
        cmd += ["-DON_DEVICE", "-gencode", "arch=compute_103a,code=sm_103a"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 mismatches" in out.stdout


def test_split_bits_matches_split_on_the_host(tmp_path):
    _run(tmp_path, device=False)


@pytest.mark.gpu
def test_split_bits_matches_split_on_the_device(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _run(tmp_path, device=True)

"""The integer slicing of the tensor-core FP64 GEMM (gpp_ozaki_split.cuh),
compiled for the host from the same header the kernels use: for doubles of
every magnitude, sign and subnormal, and chunk exponents e with |x| < 2^e,
the slices reconstruct x = 2^e sum_i s_i 2^(-7 i) to within 2^(e - 57)
(checked exactly, in 128-bit integers), s_1 lies in [-128, 128] and the others
in [-64, 63] (the bounds the exact group sums rest on), and every slice is an
integer that bf16 holds exactly.  The group table of gpp_ozaki.cu is checked
against those bounds: each group's worst-case sum over 512 k values stays
within 2^24, where FP32 accumulation is exact, and the groups stored in pairs
as one integer stay within int32.
"""
import os
import re
import shutil
import subprocess

import pytest

from conftest import REPO

CSRC = os.path.join(REPO, "doe-csfg-hackathon_gb300", "csrc")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include "gpp_ozaki_split.cuh"

static unsigned long long st = 31;
static unsigned long long nx() {
    unsigned long long z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main() {
    int bad = 0;
    const int n = 2000000;
    for (int t = 0; t < n; ++t) {
        double x;
        unsigned long long u = nx();
        switch (t % 4) {
            case 0: x = ldexp((double)(u >> 11) / 9007199254740992.0, (int)(nx() % 80) - 40); break;
            case 1: memcpy(&x, &u, 8); if (!std::isfinite(x)) x = 1.0; break;  // any finite double
            case 2: x = ldexp(1.0, (int)(nx() % 2000) - 1000) * ((u & 1) ? 1 : -1); break;
            default: x = ldexp((double)(u % 1000003), -1074 + (int)(nx() % 40)); break;  // subnormals
        }
        if (u & 2) x = -x;
        int e = 0;
        if (x != 0.0) frexp(x, &e);
        e += (int)(nx() % 3);  // the chunk's exponent may exceed this value's
        int d[gpp::kOzSlices];
        gpp::oz_slices(x, e, d);
        // sum_i d_i 2^(7 (S - i)) vs x 2^(7 S - e), exactly: x = m 2^ex.
        __int128 sum = 0;
        for (int i = 0; i < gpp::kOzSlices; ++i) {
            const int lo = i == 0 ? -128 : -64, hi = i == 0 ? 128 : 63;
            if (d[i] < lo || d[i] > hi) { if (bad++ < 5) printf("digit %d = %d out of range\n", i, d[i]); }
            sum = sum * 128 + d[i];
        }
        int ex;
        const double f = frexp(fabs(x), &ex);  // |x| = f 2^ex, f in [0.5, 1)
        const long long m = (long long)ldexp(f, 53);  // |x| = m 2^(ex - 53)
        const int sh = ex - 53 + 7 * gpp::kOzSlices - e;  // x 2^(7S - e) = m 2^sh
        // |sum - sign m 2^sh| <= 1/2, compared as (2 sum - 2 sign m 2^sh) in units of 2^min(sh, 0)
        __int128 lhs = 2 * sum, rhs = (__int128)(x < 0 ? -m : m) * 2;
        if (sh >= 0) {
            rhs <<= sh;
            if (lhs != rhs) { if (bad++ < 5) printf("x %a e %d: not exact\n", x, e); }
        } else if (sh > -100) {
            lhs <<= -sh;
            __int128 diff = lhs - rhs;
            if (diff < 0) diff = -diff;
            if (diff > ((__int128)1 << -sh)) { if (bad++ < 5) printf("x %a e %d: error above half a unit\n", x, e); }
        } else if (sum != 0) {
            if (bad++ < 5) printf("x %a e %d: tiny value gave slices\n", x, e);
        }
    }
    printf("%d failures\n", bad);
    return bad ? 1 : 0;
}
"""


def test_slices_reconstruct_and_stay_in_range(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = tmp_path / "ozaki_split_check.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "ozaki_split_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", CSRC, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 failures" in out.stdout


def _table(name, text):
    m = re.search(name + r"\[(?:kPairs|kGroups|kSlots)\] = \{([^}]*)\}", text)
    return [int(v) for v in m.group(1).replace("\n", " ").split(",")]


def test_group_table_sums_fit_in_fp32_and_pairs_in_int32():
    """Each group's worst-case sum over a chunk stays within 2^24 (exact FP32
    accumulation in tensor memory); the groups stored in pairs as one integer
    (the even group times 2^shift plus the odd one, scale 2^(-7 d) of the odd
    group) stay below 2^31, and the combining pass's split of that integer
    into 128 (v >> 7) and v & 127 gives two floats that hold it exactly."""
    text = open(os.path.join(CSRC, "gpp_ozaki.cu")).read()
    pi, pj, end = _table("kPairI", text), _table("kPairJ", text), _table("kGroupEnd", text)
    slot_d, slot_shift = _table("kSlotD", text), _table("kSlotShift", text)
    kc = int(re.search(r"constexpr int kKcMax = (\d+);", text).group(1))
    bound = lambda i: 128 if i == 1 else 64
    pairs = set(zip(pi, pj))
    # every pair with i + j <= S + 1 exactly once, none beyond
    assert len(pairs) == len(pi) == 36
    assert pairs == {(i, j) for i in range(1, 9) for j in range(1, 9) if i + j <= 9}
    groups, cur = [], []
    for i, j, e in zip(pi, pj, end):
        cur.append((i, j))
        if e:
            groups.append(cur)
            cur = []
    assert not cur and len(groups) == 10 and len(slot_d) == len(slot_shift) == 5
    gd, worst = [], []
    for g in groups:
        d = {i + j for i, j in g}
        assert len(d) == 1
        gd.append(d.pop())
        worst.append(sum(bound(i) * bound(j) for i, j in g) * kc)
        assert worst[-1] <= 2 ** 24
    for s, (d, sh) in enumerate(zip(slot_d, slot_shift)):
        de, do = gd[2 * s], gd[2 * s + 1]
        assert do == d and (do - de) * 7 == sh  # the even group's weight relative to the odd
        packed = (worst[2 * s] << sh) + worst[2 * s + 1]
        assert packed < 2 ** 31
        assert (packed >> 7) <= 2 ** 24  # 128 (v >> 7) is an exact float


HELPERS = r"""
#include <cfenv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include "gpp_ozaki_split.cuh"

static unsigned long long st = 77;
static unsigned long long nx() {
    unsigned long long z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double any_double(int t) {
    unsigned long long u = nx();
    double x;
    switch (t % 5) {
        case 0: x = ldexp((double)(u >> 11) / 9007199254740992.0, (int)(nx() % 80) - 40); break;
        case 1: memcpy(&x, &u, 8); if (!std::isfinite(x)) x = 1.5; break;
        case 2: x = ldexp((double)(u % 1000003), -1074 + (int)(nx() % 60)); break;  // subnormal
        case 3: x = ldexp(1.0, (int)(nx() % 2046) - 1022); break;                   // powers of two
        default: x = ldexp(1.0 - ldexp(1.0, -53), 1024 - (int)(nx() % 3)); break;   // near the top
    }
    return (nx() & 1) ? -x : x;
}

int main() {
    int bad = 0;
    volatile double vx, vy;
    for (int t = 0; t < 2000000; ++t) {
        const double x = any_double(t), y = (t & 8) ? any_double(t / 7) : x * ldexp(1.0, (int)(nx() % 9) - 4);
        const unsigned long long b = gpp::oz_sum_abs_bits(x, y);
        vx = fabs(x);
        vy = fabs(y);
        if (std::signbit(x) != std::signbit(y)) {
            if (b != 0) { if (bad++ < 5) printf("opposite signs gave %llx\n", b); }
            continue;
        }
        fesetround(FE_UPWARD);
        const double up = vx + vy;  // the smallest double >= |x| + |y| (Inf past the top)
        fesetround(FE_TONEAREST);
        const double B = gpp::oz_double(b);
        // B >= the exact sum, so B >= up; and no more than one unit above it
        if (!(B >= up) || (std::isfinite(up) && B > nextafter(up, INFINITY))) {
            if (bad++ < 5) printf("x %a y %a: bound %a, sum rounded up %a\n", x, y, B, up);
        }
    }
    for (int t = 0; t < 2000000; ++t) {
        double v;
        switch (t % 4) {
            case 0: v = ldexp((double)(nx() >> 11) / 9007199254740992.0 + 0.5, (int)(nx() % 200) - 100); break;
            case 1: v = ldexp(1.0, (int)(nx() % 200) - 100) * (1.0 - ldexp((double)(nx() % 64), -40)); break;
            case 2: v = ldexp(1.0, (int)(nx() % 200) - 100) * (1.0 + ldexp((double)(nx() % 64), -50)); break;
            default: v = ldexp(1.0, (int)(nx() % 200) - 100); break;
        }
        if (nx() & 1) v = -v;
        const float h = (float)v;
        const float l = (float)(v - (double)h);  // |l| <= ulp(h) / 2: a normalised pair
        bool ok = false;
        const double d = gpp::oz_pair_to_double(h, l, &ok);
        const long double want = (long double)h + (long double)l;
        const double ulp = fabs(nextafter((double)want, INFINITY) - (double)want);
        if (!ok || fabsl((long double)d - want) > ulp) {
            if (bad++ < 5) printf("h %a l %a: got %a want %La (ok %d)\n", h, l, d, want, (int)ok);
        }
    }
    bool ok = true;
    const double z = gpp::oz_pair_to_double(-0.0f, 0.0f, &ok);
    if (!ok || z != 0.0 || !std::signbit(z)) { ++bad; printf("signed zero\n"); }
    gpp::oz_pair_to_double(1e-40f, 0.0f, &ok);
    if (ok) { ++bad; printf("subnormal head not refused\n"); }
    printf("%d failures\n", bad);
    return bad ? 1 : 0;
}
"""


def test_fp64_free_helpers_bound_and_assemble(tmp_path):
    """The bit-level steps that keep FP64 instructions out of the exponent
    and combining passes: the bound on |x + y| is never below the sum (so no
    slice overflows) and at most one unit above it rounded up; a normalised
    float-float pair assembles into a double within one unit in the last
    place of h + l."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = tmp_path / "ozaki_helpers_check.cu"
    src.write_text(HELPERS)
    exe = tmp_path / "ozaki_helpers_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-Xcompiler", "-frounding-math", "-I", CSRC, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 failures" in out.stdout

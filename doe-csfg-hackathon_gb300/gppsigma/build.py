"""Build recipe of libgpp_gb300.so (sm_103a only, in-tree).

Each translation unit of ``csrc/`` is compiled in parallel with nvcc for
``compute_103a/sm_103a`` and linked into ``gppsigma/_lib/libgpp_gb300.so``;
``gpp_driver.ex`` (a C++ host program that calls the kernels through the
reference's own entry-point signatures) is linked next to it.  No cmake, no
torch extension machinery: plain nvcc, so the same recipe runs on x86 and on
the Arm GPU hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # doe-csfg-hackathon_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(ROOT, "_build")
LIB = os.path.join(LIBDIR, "libgpp_gb300.so")
DRIVER = os.path.join(LIBDIR, "gpp_driver.ex")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["gpp_api.cu", "gpp_fp64.cu", "gpp_mixed.cu", "gpp_batched.cu", "gpp_static.cu",
               "gpp_gemm.cu", "gpp_gemm_mixed.cu", "gpp_ozaki.cu", "gpp_compat.cpp"]
DRIVER_SOURCES = ["gpp_driver.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 kernels cannot be built")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _compile(src: str, obj: str, extra: list[str]) -> None:
    cmd = [_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", INCLUDE, "-I", CSRC, *extra, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA/C++ source and link libgpp_gb300.so (+ driver)."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    headers = _headers()
    jobs = []
    for name in LIB_SOURCES + DRIVER_SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJDIR, name + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o, []) for s, o in jobs]
            for f in futs:
                f.result()
    lib_objs = [os.path.join(OBJDIR, n + ".o") for n in LIB_SOURCES]
    if force or _stale(LIB, lib_objs):
        # Every kernel is this library's own: it links the CUDA runtime only.
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *lib_objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    drv_objs = [os.path.join(OBJDIR, n + ".o") for n in DRIVER_SOURCES]
    if force or _stale(DRIVER, drv_objs + [LIB]):
        cmd = [_nvcc(), *ARCH, "-o", DRIVER + ".tmp", *drv_objs, "-L", LIBDIR, "-lgpp_gb300",
               "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(DRIVER + ".tmp", DRIVER)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)

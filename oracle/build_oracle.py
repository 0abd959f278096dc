"""Build recipe for the oracle -- TEST INFRASTRUCTURE ONLY.

Two products:

* ``oracle/_build/libgpp_oracle.so`` -- the C restatement (gpp_oracle.c),
  compiled with ``-ffp-contract=off`` so x86 and Arm hosts give the same bits.
  Built wherever the tests or the benchmark's CPU leg run.
* ``oracle/_ref/`` -- the reference's own sequential code, compiled from its
  sources where they lie (only where the reference checkout is present; it is
  never copied into this repository):
    - ``libref_complex_seq.so``: gppComplex_seq.cpp + ref_harness.cpp
    - ``libref_kerseq.so``:      gppKerSeq.cpp      + ref_harness.cpp
    - ``gppKerSeq.ex``, ``gppComplex_seq.ex``, ``gppOpenMP3.ex``: the
      unmodified reference executables (README known-answer runs, CPU timing).
    - ``src/gppOpenMP3.cpp``: an untracked copy of the reference's OpenMP
      program, a single self-contained source file, staged here so that a
      host without the reference checkout (the GPU host, an aarch64 machine
      that cannot run the x86 executable built here) compiles the unmodified
      program itself (``build_openmp_reference``) for bench.py's reference
      arm.  oracle/_ref/ is git-ignored: nothing of the reference is committed.
    - ``GPPComplex.cubin`` and ``gppCuda.cubin``: the device code of the
      reference's two CUDA versions (GPPComplex.cu, called by gppCudaVer.cpp;
      gppCuda.cu, the unified-memory one) for sm_103a, loaded by
      oracle/ref_gpu.py to time the reference's GPU kernels beside the new
      ones.  Device code has no host architecture, so it runs on the GPU host
      as built here.  gppCuda.cu compiles with cuda13_prefetch_shim.h
      force-included (an overload of the pre-CUDA-13 cudaMemPrefetchAsync).
  The reference's main() is renamed with -Dmain=... in the library builds.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout (read-only); GPP_REFERENCE_DIR overrides the default.
DEFAULT_REF_DIR = os.environ.get("GPP_REFERENCE_DIR", "/root/reference")
STAGE = os.path.join(REF_OUT, "src")
OPENMP_EX = os.path.join(REF_OUT, "gppOpenMP3.ex")

ORACLE_SO = os.path.join(BUILD, "libgpp_oracle.so")


def _run(cmd: list[str]) -> None:
    subprocess.run(cmd, check=True)


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement into oracle/_build/libgpp_oracle.so."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "gpp_oracle.c"), os.path.join(HERE, "gpp_oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        base = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
                os.path.join(HERE, "gpp_oracle.c"), "-o", ORACLE_SO + ".tmp", "-lm"]
        try:
            _run(base[:1] + ["-fopenmp"] + base[1:])
        except subprocess.CalledProcessError:
            _run(base)  # no OpenMP runtime on this host: single-threaded oracle
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_reference(ref_dir: str = DEFAULT_REF_DIR, force: bool = False) -> bool:
    """Compile the reference's own CPU code into oracle/_ref/ (returns False
    when the reference sources are not present on this machine)."""
    if not os.path.isfile(os.path.join(ref_dir, "gppComplex_seq.cpp")):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    harness = os.path.join(HERE, "ref_harness.cpp")
    common = ["g++", "-O3", "-ffp-contract=off", "-fPIC", "-w", "-I", ref_dir, "-I", HERE]
    libs = [("libref_complex_seq.so", "gppComplex_seq.cpp", "REF_COMPLEX_SEQ"),
            ("libref_kerseq.so", "gppKerSeq.cpp", "REF_KERSEQ")]
    for out, src, macro in libs:
        target = os.path.join(REF_OUT, out)
        srcp = os.path.join(ref_dir, src)
        if force or _stale(target, [srcp, harness]):
            _run(common + ["-shared", "-D" + macro, "-Dmain=gpp_reference_unused_main",
                           srcp, harness, "-o", target])
    os.makedirs(STAGE, exist_ok=True)
    staged = os.path.join(STAGE, "gppOpenMP3.cpp")
    if force or _stale(staged, [os.path.join(ref_dir, "gppOpenMP3.cpp")]):
        shutil.copyfile(os.path.join(ref_dir, "gppOpenMP3.cpp"), staged)
    exes = [("gppKerSeq.ex", "gppKerSeq.cpp", []),
            ("gppComplex_seq.ex", "gppComplex_seq.cpp", []),
            ("gppOpenMP3.ex", "gppOpenMP3.cpp", ["-fopenmp"])]
    for out, src, extra in exes:
        target = os.path.join(REF_OUT, out)
        srcp = os.path.join(ref_dir, src)
        if force or _stale(target, [srcp]):
            _run(["g++", "-O3", "-w", "-I", ref_dir] + extra + [srcp, "-o", target])
    build_reference_cubin(ref_dir, force)
    return True


def build_openmp_reference(ref_dir: str = DEFAULT_REF_DIR, force: bool = False) -> str | None:
    """Compile the reference's unmodified OpenMP program (gppOpenMP3.cpp, with
    the reference's own -O3 -fopenmp) into oracle/_ref/gppOpenMP3.ex, from the
    checkout when present, else from the staged copy in oracle/_ref/src/.
    Returns the executable's path, or None when neither source is here or
    the host has no OpenMP compiler."""
    src = os.path.join(ref_dir, "gppOpenMP3.cpp")
    if not os.path.isfile(src):
        src = os.path.join(STAGE, "gppOpenMP3.cpp")
    if not os.path.isfile(src):
        return OPENMP_EX if _runs(OPENMP_EX) else None
    if force or _stale(OPENMP_EX, [src]) or not _runs(OPENMP_EX):
        os.makedirs(REF_OUT, exist_ok=True)
        try:
            _run(["g++", "-O3", "-w", "-fopenmp", src, "-o", OPENMP_EX + ".tmp"])
        except (subprocess.CalledProcessError, OSError):
            return None
        os.replace(OPENMP_EX + ".tmp", OPENMP_EX)
    return OPENMP_EX


def _runs(exe: str) -> bool:
    """Whether `exe` exists and runs on this host (it prints its usage line
    and exits when given no arguments)."""
    if not os.path.isfile(exe):
        return False
    try:
        subprocess.run([exe], capture_output=True, timeout=30)
        return True
    except (OSError, subprocess.TimeoutExpired):
        return False


def build_reference_cubin(ref_dir: str = DEFAULT_REF_DIR, force: bool = False) -> bool:
    """Compile the reference's CUDA kernels (device code only) into
    oracle/_ref/{GPPComplex,gppCuda}.cubin; False without the sources or nvcc."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.isfile(os.path.join(ref_dir, "GPPComplex.cu")) or not os.path.exists(nvcc):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    shim = os.path.join(HERE, "cuda13_prefetch_shim.h")
    # GPPComplex.cu with the reference's own device flags (Makefile.cuda:9-10),
    # its sm_30 target replaced by sm_103a; gppCuda.cu has no build line in
    # the reference, so plain -O3.
    jobs = [("GPPComplex.cubin", "GPPComplex.cu", ["--maxrregcount=150"],
             [os.path.join(ref_dir, "GPPComplex.h")]),
            ("gppCuda.cubin", "gppCuda.cu", ["-include", shim], [shim])]
    for out, src, extra, deps in jobs:
        srcp = os.path.join(ref_dir, src)
        target = os.path.join(REF_OUT, out)
        if force or _stale(target, [srcp] + deps):
            _run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w",
                  "-I", ref_dir] + extra + [srcp, "-o", target + ".tmp"])
            os.replace(target + ".tmp", target)
    return True


def main() -> int:
    build_oracle(force="--force" in sys.argv)
    ok = build_reference(force="--force" in sys.argv)
    omp = build_openmp_reference(force="--force" in sys.argv)
    print("reference OpenMP program:", omp or "not available on this host")
    print("oracle:", ORACLE_SO)
    print("reference:", REF_OUT if ok else "not present on this machine")
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Drop-in check: the reference's own CUDA host driver (gppCudaVer.cpp,
unmodified) compiles for sm_103a and links against libgpp_gb300.so in place of
the reference's GPPComplex.o, so every entry point it calls resolves to the
GB300 implementation.  Needs the reference checkout (compile + link only)."""
import os
import subprocess

import pytest

from gppsigma import build

# The reference checkout, read-only (oracle/build_oracle.py resolves
# GPP_REFERENCE_DIR the same way).
import build_oracle  # noqa: E402

REF = build_oracle.DEFAULT_REF_DIR


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "gppCudaVer.cpp")),
                    reason="reference checkout not present")
def test_reference_driver_links_against_library(tmp_path):
    lib = build.build()
    nvcc = build._nvcc()
    obj = tmp_path / "gppCudaVer.o"
    exe = tmp_path / "gppCudaVer.ex"
    subprocess.run([nvcc, *build.ARCH, "-O3", "-w", "-Xcompiler", "-fopenmp", "-I", REF, "-c",
                    os.path.join(REF, "gppCudaVer.cpp"), "-o", str(obj)], check=True)
    undef = subprocess.run(["nm", "-C", "--undefined-only", str(obj)], capture_output=True,
                           text=True, check=True).stdout
    assert "d_till_nvband(" in undef and "d_noFlagOCCSolver(" in undef
    subprocess.run([nvcc, *build.ARCH, str(obj), "-o", str(exe), "-L", os.path.dirname(lib),
                    "-lgpp_gb300", "-Xcompiler", "-fopenmp"], check=True)
    assert exe.exists()

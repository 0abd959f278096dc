"""The public header from plain C: include/gpp_gb300.h compiles as strict C11
with every warning an error, and a C program links against libgpp_gb300.so
and calls the entry points that need no device (argument validation, error
messages, stream and precision setters, variant names)."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO
from gppsigma import build, capi

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "gpp_gb300.h"

#define CHECK(c) do { if (!(c)) { printf("FAIL line %d: %s\n", __LINE__, #c); return 1; } } while (0)

int main(void) {
    gpp_problem p;
    gpp_outputs o;
    memset(&p, 0, sizeof p);
    memset(&o, 0, sizeof o);
    CHECK(gpp_sigma(NULL, NULL, NULL) == GPP_ERR_INVALID_ARGUMENT);
    CHECK(strstr(gpp_last_error_message(), "NULL") != NULL);
    p.number_bands = 4; p.nvband = 5; p.ncouls = 10; p.ngpown = 2; p.nw = 3;
    CHECK(gpp_sigma(&p, &o, NULL) == GPP_ERR_INVALID_ARGUMENT);
    CHECK(strstr(gpp_last_error_message(), "nvband") != NULL);
    CHECK(gpp_kernel_gpu(NULL, NULL, NULL, NULL, 10, 2, 4, NULL, NULL, NULL, NULL, 0, 3, NULL,
                         NULL) == GPP_ERR_INVALID_ARGUMENT);
    CHECK(gpp_set_stream((gpp_stream_t)0x10) == GPP_OK);
    CHECK(gpp_get_stream() == (gpp_stream_t)0x10);
    CHECK(gpp_set_stream(NULL) == GPP_OK);
    CHECK(gpp_get_dropin_precision() == GPP_PRECISION_FP64);
    CHECK(gpp_set_dropin_precision(GPP_PRECISION_MIXED) == GPP_OK);
    CHECK(gpp_get_dropin_precision() == GPP_PRECISION_MIXED);
    CHECK(gpp_set_dropin_precision(7) == GPP_ERR_INVALID_ARGUMENT);
    CHECK(gpp_set_dropin_precision(-1) == GPP_OK);
    CHECK(gpp_get_dropin_precision() == GPP_PRECISION_FP64);
    CHECK(gpp_variant_count() > 0);
    CHECK(gpp_variant_name(0) != NULL && strlen(gpp_variant_name(0)) > 0);
    printf("ok %d variants\n", gpp_variant_count());
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_is_strict_c_and_the_library_links_from_c(tmp_path):
    build.build()
    src = tmp_path / "use_gpp.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "use_gpp"
    libdir = os.path.dirname(capi.library_path())
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Wpedantic", "-Werror",
           "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-lgpp_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    env = {k: v for k, v in os.environ.items() if k != "GPP_DROPIN_PRECISION"}
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60, env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")

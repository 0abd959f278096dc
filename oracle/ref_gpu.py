"""The reference's own CUDA kernels on the GPU -- TEST AND MEASUREMENT
INFRASTRUCTURE ONLY (the "old GPU" comparison; nothing in the product calls
this).

oracle/_ref/GPPComplex.cubin and oracle/_ref/gppCuda.cubin are the device
code of the reference's two CUDA versions, compiled from its sources by
oracle/build_oracle.py where the reference checkout is present.  This module
loads them with the CUDA driver API and launches their kernels exactly as the
reference's host code does.  GPPComplex.cu (the version gppCudaVer.cpp
calls):

* d_till_nvband     (GPPComplex.cu:406-417): d_flagOCC_solver on a
  (nvband, ngpown) grid of 32-thread blocks;
* d_noFlagOCCSolver (GPPComplex.cu:421-433): d_achtempSolver on number_bands
  blocks of 2 threads;

both adding into caller-zeroed achtemp_re/achtemp_im/asxtemp/acht_n1_loc, as
gppCudaVer.cpp:389-399 calls them.  gppCuda.cu (unified memory): call_compute
on number_bands*ngpown/256 blocks of 256 threads, one thread per (n1, my_igp)
(gppCuda.cu:376-380), adding into caller-zeroed complex achtemp/asxtemp.  The
reference kernels take the band-independent wx_array[3] (nstart = 0,
nend = 3, GPPComplex.cu:2-3, gppCuda.cu:212).  gppCuda.cu's occupied bands do
not reset scht/ssxt between frequencies (gppCuda.cu:176-185,220-224), so its achtemp
only agrees with the others when nvband = 0.

Shapes are checked before any launch against what the reference kernels
index (read from GPPComplex.cu): d_achtempSolver reads inv_igp_index[my_igp]
past ngpown when ncouls is odd (its leftover count is taken from ncouls,
GPPComplex.cu:349-353) and skips the last G' row when ngpown is odd;
d_flagOCC_solver reads column ig = threadIdx.x unguarded when ncouls <= 32
(:172-176, :198-200).  So ncouls must be even and above 32, ngpown even, nw 3,
and every inv_igp_index entry non-negative.

    python oracle/ref_gpu.py --workload production --repeat 2

prints one JSON line: the reference kernels' time and terms/s beside the new
library's drop-in entry points (FP64 and mixed) on the same device inputs,
and their achtemp difference.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "GPPComplex.cubin")
CUBIN_UNIFIED = os.path.join(HERE, "_ref", "gppCuda.cubin")
NW = 3
FLAG_THREADS = 32    # d_till_nvband, GPPComplex.cu:409
NOFLAG_THREADS = 2   # d_noFlagOCCSolver, GPPComplex.cu:424
UNIFIED_THREADS = 256  # gppCuda.cu:376


class Unavailable(RuntimeError):
    pass


def check_shape(number_bands: int, nvband: int, ncouls: int, ngpown: int, nw: int,
                inv_igp_min: int) -> None:
    """Raise ValueError unless the reference kernels stay in bounds."""
    if nw != NW:
        raise ValueError("the reference kernels compute exactly 3 frequencies")
    if ncouls % 2 or ncouls <= FLAG_THREADS:
        raise ValueError("ncouls must be even and above 32 for the reference kernels")
    if ngpown % 2 or ngpown < 2:
        raise ValueError("ngpown must be even for the reference kernels")
    if not 0 <= nvband <= number_bands:
        raise ValueError("bad nvband")
    if inv_igp_min < 0:
        raise ValueError("negative inv_igp_index entries")


class _Module:
    """A cubin loaded into the current CUDA context (the one torch uses on
    this thread), its kernels looked up by name."""

    def __init__(self, cubin: str):
        if not os.path.exists(cubin):
            raise Unavailable(f"{cubin} not built (needs the reference sources and nvcc)")
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current on this thread
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        self._ok(self.cu.cuModuleLoad(C.byref(self.mod), cubin.encode()), "cuModuleLoad")
        n = C.c_uint()
        self._ok(self.cu.cuModuleGetFunctionCount(C.byref(n), self.mod), "cuModuleGetFunctionCount")
        funcs = (C.c_void_p * n.value)()
        self._ok(self.cu.cuModuleEnumerateFunctions(funcs, n, self.mod), "cuModuleEnumerateFunctions")
        self.names = {}
        for f in funcs:
            name = C.c_char_p()
            self._ok(self.cu.cuFuncGetName(C.byref(name), C.c_void_p(f)), "cuFuncGetName")
            self.names[name.value.decode()] = C.c_void_p(f)

    def _ok(self, r: int, what: str) -> None:
        if r != 0:
            raise Unavailable(f"{what} failed with CUresult {r}")

    def _find(self, stem: str):
        hits = [f for n, f in self.names.items() if stem in n]
        if len(hits) != 1:
            raise Unavailable(f"kernel {stem} not found once in the cubin ({sorted(self.names)})")
        return hits[0]

    def _launch(self, f, grid, block, args, stream: int) -> None:
        vals = []
        for kind, v in args:
            vals.append(C.c_int(v) if kind == "i" else C.c_void_p(v))
        params = (C.c_void_p * len(vals))(*[C.cast(C.byref(v), C.c_void_p) for v in vals])
        self._ok(self.cu.cuLaunchKernel(f, C.c_uint(grid[0]), C.c_uint(grid[1]), C.c_uint(1),
                                        C.c_uint(block), C.c_uint(1), C.c_uint(1), C.c_uint(0),
                                        C.c_void_p(stream), params, None), "cuLaunchKernel")


class RefKernels(_Module):
    """GPPComplex.cu's d_flagOCC_solver and d_achtempSolver."""

    def __init__(self, cubin: str = CUBIN):
        super().__init__(cubin)
        self.flag = self._find("d_flagOCC_solver")
        self.noflag = self._find("d_achtempSolver")

    def run(self, d, out, stream: int) -> None:
        """d_till_nvband then d_noFlagOCCSolver on device inputs `d` (fields
        of gppsigma.ops.DeviceInputs, band-independent wx_array[3]); `out`
        holds zeroed achtemp_re, achtemp_im (float64 [3]), asxtemp (complex128
        [3]) and acht_n1_loc (complex128 [number_bands])."""
        p = lambda t: t.data_ptr()
        flag_args = [("p", p(out["asxtemp"])), ("p", p(d.inv_igp_index)), ("p", p(d.vcoul)),
                     ("p", p(out["acht_n1_loc"])), ("p", p(d.wtilde_array)), ("p", p(d.aqsmtemp)),
                     ("p", p(d.aqsntemp)), ("p", p(d.I_eps_array)), ("p", p(d.wx_array)),
                     ("i", d.nvband), ("i", d.ncouls), ("i", d.ngpown), ("i", FLAG_THREADS),
                     ("p", p(out["achtemp_re"])), ("p", p(out["achtemp_im"]))]
        noflag_args = [("i", d.number_bands), ("i", d.nvband), ("i", d.ngpown), ("i", d.ncouls),
                       ("p", p(d.inv_igp_index)), ("p", p(d.wx_array)), ("p", p(d.wtilde_array)),
                       ("p", p(d.aqsmtemp)), ("p", p(d.aqsntemp)), ("p", p(d.I_eps_array)),
                       ("p", p(d.vcoul)), ("p", p(out["achtemp_re"])), ("p", p(out["achtemp_im"])),
                       ("p", p(out["acht_n1_loc"])), ("i", NOFLAG_THREADS)]
        if d.nvband > 0:
            self._launch(self.flag, (d.nvband, d.ngpown), FLAG_THREADS, flag_args, stream)
        self._launch(self.noflag, (d.number_bands, 1), NOFLAG_THREADS, noflag_args, stream)


class UnifiedKernel(_Module):
    """gppCuda.cu's call_compute."""

    def __init__(self, cubin: str = CUBIN_UNIFIED):
        super().__init__(cubin)
        self.kern = self._find("call_compute")

    def run(self, d, out, stream: int) -> None:
        """call_compute on device inputs `d` (band-independent wx_array[3]);
        `out` holds zeroed complex128 achtemp and asxtemp [3].  Pairs past the
        last full block of 256 are not computed, as in the reference, so
        number_bands * ngpown must be a multiple of 256 for a full sum."""
        p = lambda t: t.data_ptr()
        args = [("i", d.number_bands), ("i", d.ngpown), ("i", d.nvband),
                ("p", p(d.inv_igp_index)), ("i", d.ncouls), ("p", p(d.wx_array)),
                ("p", p(d.aqsmtemp)), ("p", p(d.aqsntemp)), ("p", p(d.I_eps_array)),
                ("p", p(d.wtilde_array)), ("p", p(out["achtemp"])), ("p", p(out["asxtemp"])),
                ("p", p(d.vcoul))]
        blocks = d.number_bands * d.ngpown // UNIFIED_THREADS
        if blocks:
            self._launch(self.kern, (blocks, 1), UNIFIED_THREADS, args, stream)


def zeroed_outputs(number_bands: int):
    import torch
    f64, c128 = torch.float64, torch.complex128
    return {"achtemp_re": torch.zeros(NW, dtype=f64, device="cuda"),
            "achtemp_im": torch.zeros(NW, dtype=f64, device="cuda"),
            "achtemp": torch.zeros(NW, dtype=c128, device="cuda"),
            "asxtemp": torch.zeros(NW, dtype=c128, device="cuda"),
            "acht_n1_loc": torch.zeros(number_bands, dtype=c128, device="cuda")}


def band_independent(d):
    """The same device inputs with one wx row (the reference's wx_array[3])."""
    import dataclasses
    return dataclasses.replace(d, wx_array=d.wx_array.reshape(-1, d.nw)[:1].contiguous(),
                               wx_stride=0)


def compare(workload: str, repeat: int, seed: int, nvband: int | None = None) -> dict:
    import dataclasses
    import torch
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "doe-csfg-hackathon_gb300"))
    from gppsigma import capi, ops, workload as W
    shape = W.CONFIGS[workload]
    if nvband is not None:
        shape = dataclasses.replace(shape, nvband=nvband)
    d = band_independent(ops.device_inputs(shape, seed))
    check_shape(d.number_bands, d.nvband, d.ncouls, d.ngpown, d.nw,
                int(d.inv_igp_index.min().item()))
    ref = RefKernels()
    lib = capi.load()
    stream = torch.cuda.current_stream()
    terms = shape.terms

    def timed(fn, complex_out=False, warm=False):
        ms = []
        res = None
        if warm:  # one untimed call: workspace and library handles are set up once per process
            out = zeroed_outputs(d.number_bands)
            fn(out)
            torch.cuda.synchronize()
        for _ in range(repeat):
            out = zeroed_outputs(d.number_bands)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn(out)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            res = out
        if complex_out:
            return min(ms), res["achtemp"].cpu().numpy()
        ach = (res["achtemp_re"] + 1j * res["achtemp_im"]).cpu().numpy()
        return min(ms), ach

    def ours(out):
        ops.d_till_nvband(d.nvband, d.ngpown, d.ncouls, d.inv_igp_index, d.wx_array,
                          d.wtilde_array, d.aqsmtemp, d.aqsntemp, d.I_eps_array, out["asxtemp"],
                          d.vcoul, out["acht_n1_loc"], out["achtemp_re"], out["achtemp_im"], 1.0)
        ops.d_noFlagOCCSolver(d.number_bands, d.nvband, d.ngpown, d.ncouls, d.inv_igp_index,
                              d.wx_array, d.wtilde_array, d.aqsmtemp, d.aqsntemp, d.I_eps_array,
                              d.vcoul, out["achtemp_re"], out["achtemp_im"], out["acht_n1_loc"])

    t0 = time.perf_counter()
    ms_ref, ach_ref = timed(lambda out: ref.run(d, out, stream.cuda_stream))
    wall_ref = time.perf_counter() - t0
    uni = UnifiedKernel()
    ms_uni, ach_uni = timed(lambda out: uni.run(d, out, stream.cuda_stream), complex_out=True)
    ms_fp64, ach_fp64 = timed(ours, warm=True)
    capi.check(lib.gpp_set_dropin_precision(capi.PRECISION["mixed"]), "set precision")
    try:
        ms_mixed, ach_mixed = timed(ours, warm=True)
    finally:
        capi.check(lib.gpp_set_dropin_precision(-1), "reset precision")

    import numpy as np

    def rel(g, w):
        g2, w2 = np.concatenate([g.real, g.imag]), np.concatenate([w.real, w.imag])
        return float(np.max(np.abs(g2 - w2) / np.where(w2 == 0, 1.0, np.abs(w2))))

    return {"workload": workload + " (band-independent wx, the reference's wx_array[3])",
            "nvband": shape.nvband,
            "terms": terms, "repeat": repeat,
            "reference_gpu": {"ms": ms_ref, "terms_per_s": terms / (ms_ref * 1e-3),
                              "kernels": "GPPComplex.cu d_flagOCC_solver + d_achtempSolver",
                              "wall_s_all_repeats": wall_ref},
            "reference_gpu_unified": {"ms": ms_uni, "terms_per_s": terms / (ms_uni * 1e-3),
                                      "kernels": "gppCuda.cu call_compute"},
            "gb300_fp64_dropin": {"ms": ms_fp64, "terms_per_s": terms / (ms_fp64 * 1e-3),
                                  "speedup_vs_reference_gpu": ms_ref / ms_fp64,
                                  "speedup_vs_reference_gpu_unified": ms_uni / ms_fp64},
            "gb300_mixed_dropin": {"ms": ms_mixed, "terms_per_s": terms / (ms_mixed * 1e-3),
                                   "speedup_vs_reference_gpu": ms_ref / ms_mixed,
                                   "speedup_vs_reference_gpu_unified": ms_uni / ms_mixed},
            "max_rel_err_achtemp": {"fp64_vs_reference_gpu": rel(ach_fp64, ach_ref),
                                    "mixed_vs_reference_gpu": rel(ach_mixed, ach_ref),
                                    "fp64_vs_reference_gpu_unified": rel(ach_fp64, ach_uni),
                                    "note": "gppCuda.cu carries occupied-band sums across "
                                            "frequencies; it agrees only when nvband = 0"}}


def main() -> int:
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="production")
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--seed", type=int, default=20240607)
    ap.add_argument("--nvband", type=int, default=None, help="override the workload's nvband")
    args = ap.parse_args()
    try:
        print(json.dumps(compare(args.workload, args.repeat, args.seed, args.nvband)))
    except Unavailable as e:
        print(json.dumps({"reference_gpu": "unavailable", "why": str(e)}))
    return 0


if __name__ == "__main__":
    sys.exit(main())

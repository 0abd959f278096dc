"""GPP sigma benchmark: GPP terms/s (n1 * igp * ig * iw) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload production_near_pole] [--precision mixed|fp64]

A step is one full GPP sigma reduction (occupied + unoccupied bands, all
frequencies, deterministic reduction) over one synthetic quasiparticle state
resident in HBM.  Default workload: the mini-app's production shape
(number_bands 512, nvband 2, ncouls 32768, ngpown 1638, 3 frequencies,
per-band wx) with 1% of wtilde entries placed next to a wx value; the
headline runs the mixed-precision kernel and the line also carries the FP64
kernel's rate and the mixed-vs-FP64 error on the same inputs.

Prints ONE JSON line on rank 0.  With --impl reference it times the
reference's own OpenMP program (gppOpenMP3.cpp, unmodified, compiled on this
host by oracle/build_oracle.py) on all host cores over a bounded band sample
of the same workload shape; where that program cannot run, the oracle's
restatement of its loop.

Under torchrun (N > 1) every rank runs its own independent state (weak
scaling, no data-path collective); value = all ranks' terms / max rank time.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "doe-csfg-hackathon_gb300"))

import numpy as np  # noqa: E402

from gppsigma import dist as gdist, workload as W  # noqa: E402

METRIC = "GPP terms/s (n1*igp*ig*iw) on 1 GB300: mixed vs FP64 at <=1e-8 rel err"
SEED = 20240607
# Algorithmic work of one unoccupied term: 20 FP64 flops + 1 reciprocal, plus
# 12 flops per (n1, igp, ig) for the frequency-independent product, shared by
# the nw frequencies.
FLOPS_PER_TERM_BASE = 20.0
FLOPS_PER_TRIPLE = 12.0


def mixed_fp32_ops_per_term(nwc: int) -> float:
    """FP32 operations the mixed kernel issues per unoccupied term, counted
    from its column routine: per ig column a thread issues 44 packed
    instructions shared by its frequencies (A = aqsn*Q, A*Im(wtilde),
    Im(wtilde)^2) and 74 per frequency (Re(wdiff) 8 + renormalisation 3,
    |wdiff|^2 12, reciprocal 3, the two numerators 24, the two products by
    the reciprocal 8, the two accumulations 16), each packed instruction
    doing one FP32 operation for each of the tile's two rows."""
    return (44.0 + 74.0 * nwc) / nwc


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def profile_traffic(kernel: str, workload: str, precision: str):
    """DRAM bytes (read + write) per launch of `kernel` at `workload`, from the
    ncu launch-list summary committed in profiles/ (None when not captured)."""
    path = os.path.join(REPO, "profiles", f"launches_{workload}_{precision}.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        m = re.match(rf"\s*{kernel}\S*\s.*dram_bytes_per_launch=([0-9.eE+]+)", line)
        if m:
            return float(m.group(1))
    return None


def profile_pipe(kernel_file: str, metric: str):
    """A pipe-utilisation percentage from a committed ncu summary."""
    path = os.path.join(REPO, "profiles", kernel_file)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(metric):
            m = re.search(r"([0-9.]+)\s*%", line)
            return float(m.group(1)) if m else None
    return None


FULL_FIXTURES = os.path.join(REPO, "tests", "golden", "gpp_golden_full.json")


def errors_vs_reference_outputs(workload: str, seed: int, got: dict):
    """Max relative error per real/imaginary component of achtemp and asxtemp
    against the reference's own sequential outputs for this exact workload
    (tests/golden/gpp_golden_full.json, written by make_golden.py --full; the
    oracle gives the same bits), or None when no fixture covers it."""
    import json
    if not os.path.exists(FULL_FIXTURES):
        return None
    with open(FULL_FIXTURES) as f:
        cases = {c["name"]: c for c in json.load(f)["cases"]}
    case = cases.get(workload)
    if case is None or case["seed"] != seed or W.Shape(**case["shape"]) != W.CONFIGS[workload]:
        return None
    out = {"fixture": "tests/golden/gpp_golden_full.json:" + workload,
           "inputs_sha256": case["digest"]}
    for key in ("achtemp", "asxtemp"):
        want = np.array([complex(float.fromhex(a), float.fromhex(b)) for a, b in case[key]])
        g = np.asarray(got[key], dtype=np.complex128)
        g2, w2 = np.concatenate([g.real, g.imag]), np.concatenate([want.real, want.imag])
        out[key] = float(np.max(np.abs(g2 - w2) / np.where(w2 == 0, 1.0, np.abs(w2))))
    return out


def _reference_line(args, shape, value, ms, cores, kind, sample) -> dict:
    return {"metric": METRIC, "value": value, "unit": "terms/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)" if kind == "port" else
                    "the reference program's own ramp inputs (its timing does not depend on values)",
            "impl": "reference",
            "config": {"workload": args.workload, **shape_dict(shape)},
            "cpu_baseline": {"value": value, "unit": "terms/s", "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": value, "unit": "terms/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


_TIME_RE = re.compile(r"Time Taken \*+= *([0-9.eE+-]+) *secs")


def _run_program(exe: str, nb: int, nv: int, nc: int, npg: int, threads: int) -> float:
    """One run of the reference's OpenMP program; returns its own loop time (s)."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run([exe, str(nb), str(nv), str(nc), str(npg)], capture_output=True,
                         text=True, env=env, timeout=600, check=True).stdout
    m = _TIME_RE.search(out)
    if not m:
        raise RuntimeError("no timing line in the reference program's output")
    return float(m.group(1))


def run_reference_program(args, shape: W.Shape):
    """CPU baseline: the reference's unmodified OpenMP program (gppOpenMP3.cpp,
    its loop gppOpenMP3.cpp:274-336 timed by its own gettimeofday), built on
    this host by oracle/build_oracle.py, all host threads.  It takes argv
    `number_bands nvband ncouls nodes_per_group` (ngpown = ncouls /
    nodes_per_group) and 3 frequencies, so it covers workloads of that form;
    each step runs a band sample sized to ~ref_seconds.  None when the
    program is not available here or the workload is not of that form."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import build_oracle
    exe = build_oracle.build_openmp_reference()
    if exe is None or shape.nw != 3 or shape.ngpown == 0:
        return None
    npg = shape.ncouls // shape.ngpown
    if npg < 1 or shape.ncouls // npg != shape.ngpown:
        return None
    cores = os.cpu_count() or 1
    nv, nc, ng = shape.nvband, shape.ncouls, shape.ngpown
    # Calibrate on a few unoccupied bands, then size the sample.
    probe = nv + 8
    t = _run_program(exe, probe, nv, nc, npg, cores)
    per_band = max(t / probe, 1e-4)
    nb = int(max(nv + 1, min(shape.number_bands, args.ref_seconds / per_band)))
    times = []
    for i in range(args.warmup + args.steps):
        dt = _run_program(exe, nb, nv, nc, npg, cores)
        if i >= args.warmup:
            times.append(dt)
    terms = nb * ng * nc * 3
    ms = 1e3 * statistics.mean(times)
    value = terms / (ms * 1e-3)
    sample = (f"the unmodified reference program gppOpenMP3 (OpenMP, {cores} threads), argv "
              f"'{nb} {nv} {nc} {npg}': bands 0..{nb - 1} of the workload's shape "
              f"({terms:.3e} terms per step), its own loop timer")
    return _reference_line(args, shape, value, ms, cores, "reference", sample)


def run_reference_port(args, shape: W.Shape) -> dict:
    """CPU baseline where the reference program cannot run: its OpenMP loop
    (gppOpenMP3.cpp:278-333) restated in oracle/, all host threads, a bounded
    band sample per step."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py

    cores = oracle_py.max_threads()
    # Sample: the occupied bands plus enough unoccupied bands for ~budget_s of
    # CPU work per step (calibrated on one band).
    small = W.make_inputs(W.Shape(shape.nvband + 1, shape.nvband, shape.ncouls, shape.ngpown,
                                  shape.nw, shape.dw, near_pole=shape.near_pole), SEED)
    t0 = time.perf_counter()
    oracle_py.run(small, impl="oracle_omp", nthreads=cores, band_begin=shape.nvband,
                  band_end=shape.nvband + 1)
    per_band = max(time.perf_counter() - t0, 1e-3)
    budget_s = args.ref_seconds
    nb_sample = int(max(1, min(shape.number_bands - shape.nvband, budget_s / per_band)))
    samp = W.make_inputs(W.Shape(shape.nvband + nb_sample, shape.nvband, shape.ncouls,
                                 shape.ngpown, shape.nw, shape.dw, near_pole=shape.near_pole), SEED)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle_py.run(samp, impl="oracle_omp", nthreads=cores)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    terms = samp.shape.terms
    ms = 1e3 * statistics.mean(times)
    value = terms / (ms * 1e-3)
    sample = (f"oracle restatement of the reference's OpenMP loop, bands "
              f"0..{samp.shape.number_bands - 1} ({shape.nvband} occupied + {nb_sample} "
              f"unoccupied) of the workload: {terms:.3e} terms per step")
    return _reference_line(args, shape, value, ms, cores, "port", sample)


def run_reference(args, shape: W.Shape) -> dict:
    """The reference arm: the reference's own OpenMP program where it runs on
    this host, else the oracle's restatement of its loop."""
    line = None
    try:
        line = run_reference_program(args, shape)
    except (subprocess.SubprocessError, RuntimeError, OSError) as e:
        print(f"reference program failed ({e}); timing the oracle port", file=sys.stderr)
    return line if line is not None else run_reference_port(args, shape)


def band_independent_leg(d, shape: W.Shape, steps: int) -> dict:
    """The drop-in entry points' case on the same inputs: band 0's frequencies
    for every band (the reference's wx_array[3]), so the unoccupied bands go
    through the band-sum GEMM on the tensor cores.  Per-call device time
    (CUDA events) in both precisions, with and without the per-band output:
    each call on an idle device, as the reference's program makes it (median
    of `steps`), and `steps` calls queued back to back (mean); and the error
    of each against the per-term FP64 kernel."""
    import torch
    from gppsigma import capi, ops
    lib = capi.load()
    dbi = dataclasses.replace(d, wx_array=d.wx_array.reshape(-1, shape.nw)[:1].contiguous(),
                              wx_stride=0)
    stream = torch.cuda.current_stream()

    def run(precision: str, n1: bool):
        out = ops.sigma(dbi, precision, acht_n1=n1)
        for _ in range(2):
            ops.sigma(dbi, precision, acht_n1=n1, out=out)
        ops.wait()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        single = []
        for _ in range(steps):
            torch.cuda.synchronize()
            e0.record(stream)
            ops.sigma(dbi, precision, acht_n1=n1, out=out)
            e1.record(stream)
            ops.wait()
            torch.cuda.synchronize()
            single.append(e0.elapsed_time(e1))
        e0.record(stream)
        for _ in range(steps):
            ops.sigma(dbi, precision, acht_n1=n1, out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        ops.wait()
        return out.achtemp.cpu().numpy(), float(np.median(single)), e0.elapsed_time(e1) / steps

    legs, outs = {}, {}
    for precision in ("fp64", "mixed"):
        for n1 in (False, True):
            key = precision + ("_with_per_band_output" if n1 else "")
            outs[key], ms, ms_b2b = run(precision, n1)
            legs[key] = {"ms_per_call": ms, "terms_per_s": shape.terms / (ms * 1e-3),
                         "ms_per_call_back_to_back": ms_b2b}
    capi.check(lib.gpp_set_gemm_path(0), "gpp_set_gemm_path")
    try:
        want = ops.sigma(dbi, "fp64")
        ops.wait()
        want = want.achtemp.cpu().numpy()
    finally:
        capi.check(lib.gpp_set_gemm_path(-1), "gpp_set_gemm_path")
    w2 = np.concatenate([want.real, want.imag])
    for key, got in outs.items():
        g2 = np.concatenate([got.real, got.imag])
        legs[key]["achtemp_max_rel_err_vs_per_term_fp64"] = float(
            np.max(np.abs(g2 - w2) / np.where(w2 == 0, 1.0, np.abs(w2))))
    return {"wx": "band 0's frequencies for every band (the reference's wx_array[3])",
            "band_sum": "tcgen05 tensor-core GEMM, operands cut into exact bf16 integer slices",
            "steps": steps, **legs}


def shape_dict(s: W.Shape) -> dict:
    return {"number_bands": s.number_bands, "nvband": s.nvband, "ncouls": s.ncouls,
            "ngpown": s.ngpown, "nw": s.nw, "near_pole_fraction": s.near_pole,
            "terms": s.terms}


BATCHED = {"batched64": 1.0, "batched64_half": 0.5, "batched64_quarter": 0.25}


def run_batched(args, ws, rank, local) -> int:
    """Many uneven states (number_bands ~ U{256..2048}, ncouls ~ U{8192..65536},
    ngpown = ncouls/20, nvband ~ U{2..8}, 3 frequencies; `scale` shrinks bands
    and ncouls) in one persistent launch per step, replayed from a CUDA graph.
    A step is one full run over all states."""
    import ctypes as C
    import torch
    from gppsigma import capi, ops

    torch.cuda.set_device(local)
    lib = capi.load()
    shapes = W.batched_shapes(64, SEED, scale=BATCHED[args.workload])
    devs = [ops.device_inputs(s, gdist.state_seed(SEED, rank) + i) for i, s in enumerate(shapes)]
    terms = sum(s.terms for s in shapes)

    def plan(precision, states):
        probs = (capi.GppProblem * len(states))()
        outs = (capi.GppOutputs * len(states))()
        res = []
        for i, d in enumerate(states):
            probs[i] = ops.problem_struct(d, precision, "complex_seq", 1.0)
            a = torch.empty(3, dtype=torch.complex128, device="cuda")
            x = torch.empty(3, dtype=torch.complex128, device="cuda")
            outs[i].achtemp, outs[i].asxtemp = a.data_ptr(), x.data_ptr()
            res.append((a, x))
        h = C.c_void_p()
        capi.check(lib.gpp_batch_create(C.byref(h), probs, outs, len(states)), "gpp_batch_create")
        return h, res

    stream = torch.cuda.Stream()

    def timed(precision, steps, warmup, states):
        h, res = plan(precision, states)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                capi.check(lib.gpp_batch_run(h, stream.cuda_stream), "gpp_batch_run")
            stream.synchronize()
            lib.gpp_reset_launch_count()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                capi.check(lib.gpp_batch_run(h, stream.cuda_stream), "gpp_batch_run")
            e1.record(stream)
            stream.synchronize()
        launches = lib.gpp_launch_count()
        lib.gpp_batch_destroy(h)
        return res, e0.elapsed_time(e1) / steps, launches

    clocks = ClockSampler(local)
    clocks.start()
    res, ms, launches = timed("mixed", args.steps, args.warmup, devs)
    clk = clocks.stop()
    line = {"metric": METRIC, "value": ws * terms / (ms * 1e-3), "unit": "terms/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32x2+f64", "data": "synthetic (seeded SplitMix64, reference distributions)",
            "config": {"workload": args.workload, "states": len(shapes), "terms": terms,
                       "scale": BATCHED[args.workload], "precision": "mixed",
                       "launch": "persistent work queue, CUDA graph replay",
                       "l2": "inputs larger than L2 (129 MB)"},
            "gpu_launches": int(launches), "clocks": clk}
    if args.fp64_steps > 0:
        # The FP64 leg over the first --fp64-states states (all by default;
        # at full scale one FP64 step of all 64 takes minutes), labelled.
        k = len(devs) if args.fp64_states <= 0 else min(args.fp64_states, len(devs))
        sub = devs[:k]
        sub_terms = sum(shapes[i].terms for i in range(k))
        r64, ms64, _ = timed("fp64", args.fp64_steps, args.fp64_warmup, sub)
        errs_a, errs_x = [], []

        def rel(g, w):
            g = torch.view_as_real(g).flatten().cpu().numpy()
            w = torch.view_as_real(w).flatten().cpu().numpy()
            return float(np.max(np.abs(g - w) / np.where(w == 0, 1.0, np.abs(w))))
        for (a, x), (a64, x64) in zip(res[:k], r64):
            errs_a.append(rel(a, a64))
            errs_x.append(rel(x, x64))
        line["fp64"] = {"value": ws * sub_terms / (ms64 * 1e-3), "ms_per_step": ms64,
                        "states": k, "terms": sub_terms,
                        "max_rel_err_mixed_vs_fp64": {"achtemp": max(errs_a),
                                                      "asxtemp": max(errs_x)},
                        "per_state_max_rel_err_achtemp": errs_a}
        line["mixed_speedup_vs_fp64"] = line["value"] / line["fp64"]["value"]
    if rank == 0:
        print(json.dumps(line))
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="production_near_pole",
                    choices=sorted(W.CONFIGS) + sorted(BATCHED))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--fp64-warmup", type=int, default=1,
                    help="untimed FP64-leg calls after the first (0 for the 32-frequency sweep)")
    ap.add_argument("--fp64-states", type=int, default=0,
                    help="batched workloads: time the FP64 leg on the first K states (0: all)")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="end-to-end calls timed (0: max(5, steps // 2))")
    ap.add_argument("--ref-seconds", type=float, default=4.0,
                    help="CPU seconds per step of the reference arm's band sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--bi-steps", type=int, default=5,
                    help="timed calls per leg of the band-independent-frequency report "
                         "(0: skip it)")
    ap.add_argument("--shard", default="states", choices=["states", "rows"],
                    help="states: one independent state per rank (weak scaling); rows: one "
                         "state split by G' rows across the ranks, partial sums added on "
                         "rank 0 (strong scaling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    ws, rank, local = gdist.env()
    if args.workload in BATCHED:
        return run_batched(args, ws, rank, local)
    shape = W.CONFIGS[args.workload]

    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, shape)))
        return 0

    import torch
    from gppsigma import capi, ops

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl")
        dist = dist_mod
    lib = capi.load()

    full_shape = shape
    if args.shard == "rows":
        # One state, G' rows split across the ranks (gppMPIOpenMP3.cpp:171-172).
        # Each rank generates and holds only its rows of I_eps / wtilde.
        d, (r0, r1) = gdist.rank_rows_inputs(shape, SEED, rank, ws)
        shape = dataclasses.replace(shape, ngpown=r1 - r0)
        job_terms = full_shape.terms
    else:
        d = ops.device_inputs(shape, gdist.state_seed(SEED, rank))
        job_terms = ws * shape.terms
    stream = torch.cuda.current_stream()
    input_gb = sum(getattr(d, k).numel() * getattr(d, k).element_size()
                   for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul",
                             "inv_igp_index", "wx_array")) / 1e9
    nterms = shape.terms
    unocc_terms = (shape.number_bands - shape.nvband) * shape.ngpown * shape.ncouls * shape.nw

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(precision: str, steps: int, warmup: int):
        out = ops.sigma(d, precision)
        for _ in range(warmup):
            ops.sigma(d, precision, out=out)
        ops.wait()
        barrier()
        lib.gpp_reset_launch_count()
        lib.gpp_enable_kernel_timing(1)
        kern_ms = []
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            ops.sigma(d, precision, out=out)
            if steps <= 64:
                import ctypes as C
                f = C.c_float()
                if lib.gpp_last_kernel_ms(C.byref(f)) == 0:
                    kern_ms.append(f.value)
        e1.record(stream)
        barrier()
        lib.gpp_enable_kernel_timing(0)
        launches = lib.gpp_launch_count()
        ops.wait()
        ms = gdist.max_over_ranks(e0.elapsed_time(e1) / steps, dist, "cuda")
        return out, ms, kern_ms, launches

    fp64_peak, fp32_peak = 0.0, 0.0
    if rank == 0:
        import ctypes as C
        a, b = C.c_double(), C.c_double()
        capi.check(lib.gpp_probe_fma_peaks(C.byref(a), C.byref(b)), "probe")
        fp64_peak, fp32_peak = a.value, b.value

    precision = args.precision
    variant = None
    if precision == "mixed":
        # Pick the mixed kernel's pipeline variant on this GPU (outside the
        # timed region), as a user would once per shape class.
        try:
            v = ops.autotune(d, max_bands=24)
            variant = {"index": v, "name": ops.variant_names()[v]}
        except capi.GppError:
            variant = None
    clocks = ClockSampler(local)
    clocks.start()
    res, ms, kern_ms, launches = timed(precision, args.steps, args.warmup)
    clk = clocks.stop()

    fp64_leg = None
    mixed_vs_oracle = None
    if precision == "mixed":
        r64, ms64, k64, _ = timed("fp64", args.fp64_steps, args.fp64_warmup)
        a, b = res.achtemp.cpu().numpy(), r64.achtemp.cpu().numpy()
        x, y = res.asxtemp.cpu().numpy(), r64.asxtemp.cpu().numpy()

        def rel(g, w):
            g2, w2 = np.concatenate([g.real, g.imag]), np.concatenate([w.real, w.imag])
            return float(np.max(np.abs(g2 - w2) / np.where(w2 == 0, 1.0, np.abs(w2))))
        if args.shard == "rows":
            # The one exchange step: per-rank partial sums added in rank order.
            a = gdist.sum_in_rank_order(a, dist, "cuda")
            b = gdist.sum_in_rank_order(b, dist, "cuda")
            x = gdist.sum_in_rank_order(x, dist, "cuda")
            y = gdist.sum_in_rank_order(y, dist, "cuda")
            if a is None:  # ranks other than 0
                a, b, x, y = (np.ones(1, np.complex128),) * 4
        k64ms = statistics.median(k64) if k64 else None
        fp64_leg = {"value": job_terms / (ms64 * 1e-3), "ms_per_step": ms64,
                    "kernel_ms": k64ms,
                    "max_rel_err_mixed_vs_fp64": {"achtemp": rel(a, b), "asxtemp": rel(x, y)}}
        # Both precisions against the reference's own outputs on these inputs
        # (rank 0's state is the seeded workload; with --shard rows the sums
        # above already cover the whole state).
        seed0 = SEED if args.shard == "rows" else gdist.state_seed(SEED, 0)
        if rank == 0:
            vs_ref = errors_vs_reference_outputs(args.workload, seed0, {"achtemp": a, "asxtemp": x})
            if vs_ref:
                mixed_vs_oracle = vs_ref
                fp64_leg["max_rel_err_vs_oracle"] = errors_vs_reference_outputs(
                    args.workload, seed0, {"achtemp": b, "asxtemp": y})
        if k64ms and fp64_peak:
            # The FP64 kernel against the measured FP64 FMA rate (algorithmic flops).
            a64 = unocc_terms * (FLOPS_PER_TERM_BASE + FLOPS_PER_TRIPLE / shape.nw) / (k64ms * 1e-3)
            fp64_leg["roofline"] = {"bound": "fp64", "achieved": a64 * 1e-12, "peak": fp64_peak,
                                    "unit": "TFLOP/s", "frac": a64 * 1e-12 / fp64_peak,
                                    "kernel": "noflag_fp64_kernel"}

    # End to end through the host-buffer C-ABI call: pinned host inputs
    # (which the library pulls with a kernel on the SMs, overlapped with the
    # computation), H2D + kernels + D2H every step.
    arrays = {}
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul", "inv_igp_index",
              "indinv", "wx_array"):
        src = getattr(d, k)
        host = torch.empty(src.shape, dtype=src.dtype, pin_memory=True)
        host.copy_(src)
        arrays[k] = host.numpy()
    h2d = int(sum(a.nbytes for a in arrays.values()))
    d2h = 2 * shape.nw * 16
    e2e_times, e2e_parts = [], []
    with ops.HostContext() as ctx:
        n_e2e = args.e2e_steps if args.e2e_steps > 0 else max(5, args.steps // 2)
        for i in range(2 + n_e2e):
            barrier()
            t0 = time.perf_counter()
            ctx.sigma(arrays, shape, precision)
            dt = time.perf_counter() - t0
            if i >= 2:
                e2e_times.append(dt)
                e2e_parts.append(ctx.last_timing())
    e2e_s = gdist.max_over_ranks(statistics.median(e2e_times), dist, "cuda")

    if rank != 0:
        dist.destroy_process_group()
        return 0

    # Roofline of the dominant (unoccupied-band) kernel.
    kms = statistics.median(kern_ms) if kern_ms else None
    flops = unocc_terms * (FLOPS_PER_TERM_BASE + FLOPS_PER_TRIPLE / shape.nw)
    peak = fp32_peak if precision == "mixed" else fp64_peak
    achieved = flops / (kms * 1e-3) * 1e-12 if kms else None
    kname = "mixed_noflag_kernel" if precision == "mixed" else "noflag_fp64_kernel"
    traffic = profile_traffic(kname, args.workload, precision)
    pipe_file = "ncu_noflag_mixed_profile.txt" if precision == "mixed" else "ncu_noflag_fp64_profile.txt"
    # Pipe busy cycles: a packed f32x2 instruction occupies the FMA pipe for
    # two cycles, so instruction counts understate its load.
    pipe_metric = "sm__pipe_fma_cycles_active" if precision == "mixed" else "sm__inst_executed_pipe_fp64"
    pipe_pct = profile_pipe(pipe_file, pipe_metric)
    issued = None
    if precision == "mixed" and kms and fp32_peak:
        ops = mixed_fp32_ops_per_term(shape.nw if shape.nw <= 4 else 8)
        rate = ops * unocc_terms / (kms * 1e-3)  # FP32 operations per second
        issued = {"fp32_ops_per_term": ops, "achieved_tops": rate * 1e-12,
                  "peak_tops": fp32_peak / 2.0, "frac": rate / (fp32_peak / 2.0 * 1e12),
                  "note": "issued FP32 operations (float-float emulation included) against the "
                          "measured FP32 FMA rate; 'frac' above counts algorithmic FP64-equivalent "
                          "flops only"}
    roofline = {"bound": "fp32" if precision == "mixed" else "fp64",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if (achieved and peak) else None,
                "traffic": traffic,
                "peak_source": "measured in this run: dependent-chain-free FMA probe kernel "
                               "(gpp_probe_fma_peaks), " + ("FP32" if precision == "mixed" else "FP64"),
                "flops_per_term": FLOPS_PER_TERM_BASE + FLOPS_PER_TRIPLE / shape.nw,
                "kernel": kname, "kernel_ms": kms,
                "ncu_pipe_busy_pct": pipe_pct,
                "ncu_pipe_note": f"{pipe_metric} from profiles/{pipe_file} (profile shape)",
                "traffic_note": "dram read+write bytes per launch at this workload, "
                                f"profiles/launches_{args.workload}_{precision}.txt",
                "fp64_fma_peak_tflops": fp64_peak, "fp32_fma_peak_tflops": fp32_peak}
    if issued:
        roofline["issued"] = issued

    line = {"metric": METRIC, "value": job_terms / (ms * 1e-3), "unit": "terms/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "strong" if args.shard == "rows" else "weak",
            "vs_baseline": None,
            "dtype": "f32x2+f64" if precision == "mixed" else "f64",
            "data": "synthetic (seeded SplitMix64, reference distributions)",
            "config": {"workload": args.workload, **shape_dict(full_shape), "precision": precision,
                       "mixed_variant": variant,
                       "l2": f"inputs ({input_gb:.2f} GB) larger than L2 (129 MB)",
                       "parallelism": (f"one state, G' rows split over {ws} GPU(s), partial "
                                       "sums added on rank 0 in rank order"
                                       if args.shard == "rows" else
                                       f"{ws} independent state(s), one per GPU")},
            "gpu_launches": int(launches),
            "clocks": clk,
            "e2e": {"value": job_terms / e2e_s, "unit": "terms/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                    "path": "gpp_sigma_host from pinned host buffers (median of steps)",
                    "device_ms_median": {k: statistics.median(p[k] for p in e2e_parts)
                                         for k in ("h2d_ms", "compute_ms", "d2h_ms")},
                    "wall_ms_all": [round(t * 1e3, 1) for t in e2e_times]},
            "roofline": roofline}
    if fp64_leg:
        line["fp64"] = fp64_leg
        line["mixed_speedup_vs_fp64"] = line["value"] / fp64_leg["value"]
    if mixed_vs_oracle:
        line["max_rel_err_vs_oracle"] = mixed_vs_oracle
    if rank == 0 and args.bi_steps > 0 and args.shard == "states":
        line["band_independent_wx"] = band_independent_leg(d, shape, args.bi_steps)
    if not args.no_cpu_baseline:
        ref_args = argparse.Namespace(**vars(args))
        ref_args.steps, ref_args.warmup = 1, 0
        ref = run_reference(ref_args, shape)
        line["cpu_baseline"] = ref["cpu_baseline"]
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Run the GPP sigma reduction on one synthetic workload from the command line.

    python doe-csfg-hackathon_gb300/gppsigma/run_case.py --workload profile \
        --precision mixed --repeat 3

Generates the seeded inputs, copies them to cuda:0, runs gpp_sigma `--repeat`
times (synchronising and checking device-side faults) and prints achtemp.
Useful as a fixed command line for profilers.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from gppsigma import workload as W  # noqa: E402

# Extra shapes for profiling: larger than L2 (129 MB), a few hundred MB total.
SHAPES = dict(W.CONFIGS)
SHAPES["profile"] = W.Shape(512, 2, 8192, 512, 3, near_pole=0.01)
# The 32-frequency sweep's distributions and ncouls at a fraction of its bands
# and rows (~2 GB on the device with the split planes): the 8-frequency tile.
SHAPES["sweep32_small"] = W.Shape(64, 8, 65536, 400, 32, dw=0.25)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="profile", choices=sorted(SHAPES))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--semantics", default="complex_seq", choices=["complex_seq", "kerseq"])
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--seed", type=int, default=20240607)
    ap.add_argument("--band-independent", action="store_true",
                    help="one wx row for every band (the reference's wx_array[3])")
    ap.add_argument("--acht-n1", action="store_true",
                    help="also produce the per-band output acht_n1_loc")
    ap.add_argument("--gemm-path", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="gpp_set_gemm_path mode for band-independent wx (2: FP64 GEMMs on the "
                         "FP64 pipe instead of the tensor cores)")
    args = ap.parse_args()

    import torch
    from gppsigma import capi, ops

    torch.cuda.set_device(0)
    shape = SHAPES[args.workload]
    d = ops.device_inputs(shape, args.seed)
    if args.band_independent:
        import dataclasses
        d = dataclasses.replace(d, wx_array=d.wx_array.reshape(-1, shape.nw)[:1].contiguous(),
                                wx_stride=0)
    capi.check(capi.load().gpp_set_gemm_path(args.gemm_path), "gpp_set_gemm_path")
    out = None
    for i in range(args.repeat):
        t0 = time.perf_counter()
        out = ops.sigma(d, args.precision, args.semantics, out=out, acht_n1=args.acht_n1)
        ops.wait()
        dt = time.perf_counter() - t0
        print(f"step {i}: {dt * 1e3:.2f} ms, {shape.terms / dt:.4e} terms/s")
    for iw, z in enumerate(out.achtemp.cpu().numpy()):
        print(f"achtemp[{iw}] = ({z.real:.15g},{z.imag:.15g})")
    for iw, z in enumerate(out.asxtemp.cpu().numpy()):
        print(f"asxtemp[{iw}] = ({z.real:.15g},{z.imag:.15g})")
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Generate tests/golden/gpp_golden.json from the REFERENCE's own code.

Each case is run through the reference's sequential functions (built from
gppComplex_seq.cpp / gppKerSeq.cpp into oracle/_ref/ by oracle/build_oracle.py)
on inputs from gppsigma.workload; the outputs are stored as exact hex floats
together with a sha256 digest of the generated inputs, so the fixtures pin
both the C restatement (bit-exact) and the GPU kernels (to tolerance) on any
machine, without the reference checkout.

The ramp cases are the reference's own known-answer inputs; their README
values (README.md:26-41, 15 significant digits) are stored as published.

    python tests/golden/make_golden.py         # needs the reference checkout
    python tests/golden/make_golden.py --full  # the production shapes, ~6 min each

``--full`` writes tests/golden/gpp_golden_full.json: the benchmark's own
workloads at full size (number_bands 512, nvband 2, ncouls 32768, ngpown 1638,
3 frequencies, seed 20240607; with and without 1% near-pole wtilde), summed
by the reference's functions (one thread, ~5 min per shape) and by the C
restatement on all host threads; the two must agree bit for bit before the
fixture is written.
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "doe-csfg-hackathon_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from gppsigma import workload as W  # noqa: E402
import build_oracle  # noqa: E402
import oracle_py  # noqa: E402

OUT = os.path.join(HERE, "gpp_golden.json")

# Published known answers of the reference (README.md:26-41).
README = {
    (512, 2, 800, 20): ["(-2.33321481494884e+17,-2.30534726978554e+17)",
                        "(-2.34252423351125e+17,-2.30513076345906e+17)",
                        "(-2.35188613227291e+17,-2.30484574707011e+17)"],
    (512, 2, 1600, 20): ["(-1.00387366710739e+19,-9.9815856421254e+18)",
                         "(-1.00578107032611e+19,-9.98139840041474e+18)",
                         "(-1.00769357238471e+19,-9.98115517772354e+18)"],
    (512, 2, 3200, 20): ["(-5.13842445834172e+20,-5.12423661308937e+20)",
                         "(-5.14315659139572e+20,-5.12421580271217e+20)",
                         "(-5.14789457600568e+20,-5.12418893702435e+20)"],
}

SEEDED = [
    ("small", W.CONFIGS["small"], 7),
    ("medium", W.Shape(64, 4, 4096, 256, 3), 11),
    ("single_column_row", W.Shape(6, 2, 1, 1, 3), 3),
    ("ragged", W.Shape(9, 3, 777, 13, 3), 5),
    ("all_occupied", W.Shape(5, 5, 300, 7, 3), 6),
    ("no_occupied", W.Shape(7, 0, 300, 7, 3), 8),
    ("one_frequency", W.Shape(8, 2, 500, 10, 1), 9),
    ("five_frequencies", W.Shape(8, 2, 500, 10, 5), 10),
    ("sweep32_small", W.Shape(6, 2, 256, 6, 32, dw=0.25), 12),
    ("igp_clamp", W.Shape(8, 2, 400, 12, 3, igp_overflow=3), 13),
    ("near_pole", W.Shape(16, 2, 1024, 32, 3, near_pole=0.05), 14),
    ("no_rows", W.Shape(4, 1, 100, 0, 3), 15),
]


def hexlist(a):
    if a is None:
        return None
    return [[float(z.real).hex(), float(z.imag).hex()] for z in a]


OUT_FULL = os.path.join(HERE, "gpp_golden_full.json")
# The benchmark's workloads and seed (bench.py).
FULL = [("production", 20240607), ("production_near_pole", 20240607)]


def main_full() -> int:
    """Full-size fixtures: the reference's functions and the oracle on the
    benchmark's own inputs, required to agree bit for bit."""
    cases = []
    for name, seed in FULL:
        shape = W.CONFIGS[name]
        inp = W.make_inputs(shape, seed)
        digest = inp.digest()
        ref = oracle_py.run(inp, "complex_seq", impl="ref_complex_seq")
        orc = oracle_py.run(inp, "complex_seq", impl="oracle", nthreads=oracle_py.max_threads())
        for key in ("achtemp", "asxtemp", "acht_n1_loc", "achstemp"):
            if hexlist(ref[key]) != hexlist(orc[key]):
                print(f"{name}: oracle and reference differ in {key}", file=sys.stderr)
                return 1
        cases.append({"name": name, "kind": "seeded", "shape": dataclasses.asdict(shape),
                      "seed": seed, "semantics": "complex_seq", "digest": digest,
                      "achtemp": hexlist(ref["achtemp"]), "asxtemp": hexlist(ref["asxtemp"]),
                      "acht_n1_loc": hexlist(ref["acht_n1_loc"]),
                      "achstemp": hexlist(ref["achstemp"]),
                      "oracle_bit_exact": True})
        print(name, "done", flush=True)
    with open(OUT_FULL, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --full",
                   "source": "reference functions gppComplex_seq.cpp via oracle/ref_harness.cpp; "
                             "oracle/gpp_oracle.c gives the same bits",
                   "cases": cases}, f, indent=1)
    print("wrote", OUT_FULL, len(cases), "cases")
    return 0


def main() -> int:
    build_oracle.build_oracle()
    if not build_oracle.build_reference():
        print("reference checkout not found; fixtures not regenerated", file=sys.stderr)
        return 1
    if "--full" in sys.argv:
        return main_full()
    cases = []
    for (nb, nv, nc, npg), readme in README.items():
        inp = W.ramp_inputs(nb, nv, nc, npg)
        r = oracle_py.run(inp, "kerseq", impl="ref_kerseq")
        cases.append({"name": f"ramp_{nb}_{nv}_{nc}_{npg}", "kind": "ramp",
                      "args": [nb, nv, nc, npg], "semantics": "kerseq", "digest": inp.digest(),
                      "readme_achtemp": readme, "achtemp": hexlist(r["achtemp"]),
                      "asxtemp": hexlist(r["asxtemp"]), "acht_n1_loc": hexlist(r["acht_n1_loc"]),
                      "achstemp": hexlist(r["achstemp"])})
        print(cases[-1]["name"], "done", flush=True)
    for name, shape, seed in SEEDED:
        inp = W.make_inputs(shape, seed)
        for sem in ("complex_seq", "kerseq"):
            r = oracle_py.run(inp, sem, impl="ref_" + sem)
            cases.append({"name": f"{name}_{sem}", "kind": "seeded",
                          "shape": dataclasses.asdict(shape), "seed": seed, "semantics": sem,
                          "digest": inp.digest(), "achtemp": hexlist(r["achtemp"]),
                          "asxtemp": hexlist(r["asxtemp"]),
                          "acht_n1_loc": hexlist(r["acht_n1_loc"]),
                          "achstemp": hexlist(r["achstemp"])})
            print(cases[-1]["name"], "done", flush=True)
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "source": "reference functions "
                   "gppComplex_seq.cpp / gppKerSeq.cpp via oracle/ref_harness.cpp",
                   "cases": cases}, f, indent=1)
    print("wrote", OUT, len(cases), "cases")
    return 0


if __name__ == "__main__":
    sys.exit(main())

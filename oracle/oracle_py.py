"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/libgpp_oracle.so (the C restatement, built on demand) and,
where they were built, the reference's own functions in oracle/_ref/.  Only
the tests, the smoke check and the benchmark's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

SEMANTICS = {"complex_seq": 0, "kerseq": 1}


class _Problem(C.Structure):
    _fields_ = [("number_bands", C.c_int), ("nvband", C.c_int), ("ncouls", C.c_int),
                ("ngpown", C.c_int), ("nw", C.c_int),
                ("aqsmtemp", C.c_void_p), ("aqsntemp", C.c_void_p), ("I_eps_array", C.c_void_p),
                ("wtilde_array", C.c_void_p), ("vcoul", C.c_void_p), ("inv_igp_index", C.c_void_p),
                ("wx_array", C.c_void_p), ("wx_stride", C.c_int), ("occ", C.c_double),
                ("semantics", C.c_int), ("band_begin", C.c_int), ("band_end", C.c_int)]


class _Outputs(C.Structure):
    _fields_ = [("achtemp", C.c_void_p), ("asxtemp", C.c_void_p), ("acht_n1_loc", C.c_void_p),
                ("achstemp", C.c_void_p)]


_libs: dict[str, C.CDLL] = {}


def _load(kind: str) -> C.CDLL:
    if kind in _libs:
        return _libs[kind]
    if kind == "oracle":
        lib = C.CDLL(build_oracle.build_oracle())
        for fn in (lib.oracle_sigma, lib.oracle_sigma_omp, lib.oracle_sigma_extended):
            fn.restype = C.c_int
            fn.argtypes = [C.POINTER(_Problem), C.POINTER(_Outputs), C.c_int]
        lib.oracle_max_threads.restype = C.c_int
    else:
        path = os.path.join(build_oracle.REF_OUT, f"lib{kind}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        lib.ref_sigma.restype = C.c_int
        lib.ref_sigma.argtypes = [C.POINTER(_Problem), C.POINTER(_Outputs)]
    _libs[kind] = lib
    return lib


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(build_oracle.REF_OUT, f"lib{k}.so"))
               for k in ("ref_complex_seq", "ref_kerseq"))


def max_threads() -> int:
    return _load("oracle").oracle_max_threads()


def run(inp, semantics: str = "complex_seq", nthreads: int = 1, impl: str = "oracle",
        occ: float = 1.0, band_begin: int = 0, band_end: int | None = None) -> dict:
    """Sum the GPP terms of `inp` (a gppsigma.workload.Inputs) on the CPU.

    impl: "oracle" (C restatement, sequential order), "oracle_omp" (the
    reference's OpenMP loop shape, order depends on nthreads),
    "oracle_extended" (long double with compensated sums: a reference value
    for rounding errors, not bit-comparable with the reference),
    "ref_complex_seq" / "ref_kerseq" (the reference's own functions)."""
    s = inp.shape
    nb = s.number_bands
    band_end = nb if band_end is None else band_end
    arrs = [np.ascontiguousarray(a) for a in (inp.aqsmtemp, inp.aqsntemp, inp.I_eps_array,
                                              inp.wtilde_array, inp.vcoul, inp.inv_igp_index,
                                              inp.wx_array)]
    p = _Problem()
    p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nw = nb, s.nvband, s.ncouls, s.ngpown, s.nw
    (p.aqsmtemp, p.aqsntemp, p.I_eps_array, p.wtilde_array, p.vcoul, p.inv_igp_index,
     p.wx_array) = [a.ctypes.data for a in arrs]
    wx = arrs[6]
    p.wx_stride = 0 if wx.shape[0] == 1 and nb != 1 else wx.shape[1]
    p.occ = occ
    p.semantics = SEMANTICS[semantics]
    p.band_begin, p.band_end = band_begin, band_end
    out = {"achtemp": np.zeros(s.nw, np.complex128), "asxtemp": np.zeros(s.nw, np.complex128),
           "acht_n1_loc": np.zeros(nb, np.complex128) if s.nw >= 3 else None,
           "achstemp": np.zeros(1, np.complex128)}
    o = _Outputs()
    o.achtemp, o.asxtemp = out["achtemp"].ctypes.data, out["asxtemp"].ctypes.data
    o.acht_n1_loc = out["acht_n1_loc"].ctypes.data if out["acht_n1_loc"] is not None else None
    o.achstemp = out["achstemp"].ctypes.data
    if impl == "oracle":
        rc = _load("oracle").oracle_sigma(C.byref(p), C.byref(o), nthreads)
    elif impl == "oracle_extended":
        rc = _load("oracle").oracle_sigma_extended(C.byref(p), C.byref(o), nthreads)
    elif impl == "oracle_omp":
        o.acht_n1_loc = None
        out["acht_n1_loc"] = None
        o.achstemp = None
        out["achstemp"] = None
        rc = _load("oracle").oracle_sigma_omp(C.byref(p), C.byref(o), nthreads)
    else:
        if band_begin != 0 or band_end != nb:
            raise ValueError("the reference harness sums all bands")
        rc = _load(impl).ref_sigma(C.byref(p), C.byref(o))
    if rc != 0:
        raise ValueError(f"{impl} rejected the problem (rc={rc})")
    return out

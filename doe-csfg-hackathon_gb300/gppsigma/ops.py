"""Host-side mirror of the reference's GPU operator interface, over the C ABI.

The functions named after the reference (gppKernelGPU, d_till_nvband,
d_noFlagOCCSolver, d_reduce_achstemp; GPPComplex.h:304-310) take the same
arguments in the same order, with CUDA tensors in place of raw device
pointers: complex arrays as complex128 tensors, real arrays as float64, index
arrays as int32.  Like the reference they ADD into the output tensors and run
asynchronously on the current torch stream.  Unlike the reference they raise
GppError on invalid input instead of printing.

`sigma` is the full-problem call (occupied + unoccupied bands, per-band wx,
asxtemp, precision and semantics selection); `sigma_host` runs the same call
from host (numpy) arrays through a library context, copies included.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import capi

try:
    import torch
except ImportError:  # the C ABI itself does not need torch
    torch = None


def _ptr(t, dtype, name: str, n: int | None = None) -> int:
    if t is None:
        return None
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name}: expected a torch tensor")
    if not t.is_cuda:
        raise ValueError(f"{name}: expected a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name}: expected {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name}: must be contiguous")
    if n is not None and t.numel() < n:
        raise ValueError(f"{name}: needs at least {n} elements, has {t.numel()}")
    return t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _with_stream(fn, *args):
    lib = capi.load()
    lib.gpp_set_stream(_stream())
    return fn(*args)


def gppKernelGPU(wtilde_array, aqsntemp, aqsmtemp, I_eps_array, ncouls, ngpown, number_bands,
                 wx_array, achtemp_re, achtemp_im, vcoul, nstart, nend, indinv, inv_igp_index):
    """GPPComplex.h:304: every band on the unoccupied path; adds into achtemp_re/im."""
    lib = capi.load()
    c128, f64, i32 = torch.complex128, torch.float64, torch.int32
    st = _with_stream(lib.gpp_kernel_gpu,
                      _ptr(wtilde_array, c128, "wtilde_array", ngpown * ncouls),
                      _ptr(aqsntemp, c128, "aqsntemp", number_bands * ncouls),
                      _ptr(aqsmtemp, c128, "aqsmtemp", number_bands * ncouls),
                      _ptr(I_eps_array, c128, "I_eps_array", ngpown * ncouls),
                      ncouls, ngpown, number_bands, _ptr(wx_array, f64, "wx_array", nend - nstart),
                      _ptr(achtemp_re, f64, "achtemp_re", nend - nstart),
                      _ptr(achtemp_im, f64, "achtemp_im", nend - nstart),
                      _ptr(vcoul, f64, "vcoul", ncouls), nstart, nend,
                      _ptr(indinv, i32, "indinv", ncouls),
                      _ptr(inv_igp_index, i32, "inv_igp_index", ngpown))
    capi.check(st, "gppKernelGPU")


def d_till_nvband(nvband, ngpown, ncouls, inv_igp_index, wx_array, wtilde_array, aqsmtemp,
                  aqsntemp, I_eps_array, asxtemp, vcoul, acht_n1_loc, achtemp_re, achtemp_im,
                  occ=1.0):
    """GPPComplex.cu:406: occupied bands; adds into achtemp, asxtemp, acht_n1_loc."""
    lib = capi.load()
    c128, f64, i32 = torch.complex128, torch.float64, torch.int32
    st = _with_stream(lib.gpp_till_nvband, nvband, ngpown, ncouls,
                      _ptr(inv_igp_index, i32, "inv_igp_index", ngpown),
                      _ptr(wx_array, f64, "wx_array", 3),
                      _ptr(wtilde_array, c128, "wtilde_array", ngpown * ncouls),
                      _ptr(aqsmtemp, c128, "aqsmtemp", nvband * ncouls),
                      _ptr(aqsntemp, c128, "aqsntemp", nvband * ncouls),
                      _ptr(I_eps_array, c128, "I_eps_array", ngpown * ncouls),
                      _ptr(asxtemp, c128, "asxtemp", 3), _ptr(vcoul, f64, "vcoul", ncouls),
                      _ptr(acht_n1_loc, c128, "acht_n1_loc", nvband),
                      _ptr(achtemp_re, f64, "achtemp_re", 3), _ptr(achtemp_im, f64, "achtemp_im", 3),
                      float(occ))
    capi.check(st, "d_till_nvband")


def d_noFlagOCCSolver(number_bands, nvband, ngpown, ncouls, inv_igp_index, wx_array,
                      wtilde_array, aqsmtemp, aqsntemp, I_eps_array, vcoul, achtemp_re,
                      achtemp_im, acht_n1_loc):
    """GPPComplex.cu:422: unoccupied bands; adds into achtemp and acht_n1_loc."""
    lib = capi.load()
    c128, f64, i32 = torch.complex128, torch.float64, torch.int32
    st = _with_stream(lib.gpp_noflag_occ_solver, number_bands, nvband, ngpown, ncouls,
                      _ptr(inv_igp_index, i32, "inv_igp_index", ngpown),
                      _ptr(wx_array, f64, "wx_array", 3),
                      _ptr(wtilde_array, c128, "wtilde_array", ngpown * ncouls),
                      _ptr(aqsmtemp, c128, "aqsmtemp", number_bands * ncouls),
                      _ptr(aqsntemp, c128, "aqsntemp", number_bands * ncouls),
                      _ptr(I_eps_array, c128, "I_eps_array", ngpown * ncouls),
                      _ptr(vcoul, f64, "vcoul", ncouls),
                      _ptr(achtemp_re, f64, "achtemp_re", 3), _ptr(achtemp_im, f64, "achtemp_im", 3),
                      _ptr(acht_n1_loc, c128, "acht_n1_loc", number_bands))
    capi.check(st, "d_noFlagOCCSolver")


def d_reduce_achstemp(number_bands, inv_igp_index, ncouls, aqsmtemp, aqsntemp, I_eps_array,
                      achstemp_re, achstemp_im, ngpown, vcoul):
    """GPPComplex.h:308 (declared, never defined there): reduce_achstemp over
    all bands (gppKerSeq.cpp:67-100); adds into achstemp_re[0] / achstemp_im[0]."""
    lib = capi.load()
    c128, f64, i32 = torch.complex128, torch.float64, torch.int32
    st = _with_stream(lib.gpp_reduce_achstemp_split, number_bands,
                      _ptr(inv_igp_index, i32, "inv_igp_index", ngpown), ncouls,
                      _ptr(aqsmtemp, c128, "aqsmtemp", number_bands * ncouls),
                      _ptr(aqsntemp, c128, "aqsntemp", number_bands * ncouls),
                      _ptr(I_eps_array, c128, "I_eps_array", ngpown * ncouls),
                      _ptr(achstemp_re, f64, "achstemp_re", 1), _ptr(achstemp_im, f64, "achstemp_im", 1),
                      ngpown, _ptr(vcoul, f64, "vcoul", ncouls))
    capi.check(st, "d_reduce_achstemp")


@dataclasses.dataclass
class DeviceInputs:
    """Problem arrays resident on the GPU (torch tensors)."""
    number_bands: int
    nvband: int
    ncouls: int
    ngpown: int
    nw: int
    aqsmtemp: "torch.Tensor"
    aqsntemp: "torch.Tensor"
    I_eps_array: "torch.Tensor"
    wtilde_array: "torch.Tensor"
    vcoul: "torch.Tensor"
    inv_igp_index: "torch.Tensor"
    indinv: "torch.Tensor | None"
    wx_array: "torch.Tensor"
    wx_stride: int

    def rows(self, r0: int, r1: int) -> "DeviceInputs":
        """The same problem restricted to G' rows [r0, r1) (views, no copy):
        the row sums of a sharded state, which add up to the full sums."""
        return dataclasses.replace(self, ngpown=r1 - r0, I_eps_array=self.I_eps_array[r0:r1],
                                   wtilde_array=self.wtilde_array[r0:r1],
                                   inv_igp_index=self.inv_igp_index[r0:r1])

    @classmethod
    def from_host(cls, inp, device="cuda", with_indinv: bool = True) -> "DeviceInputs":
        s = inp.shape
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
        wx = np.ascontiguousarray(inp.wx_array)
        stride = 0 if wx.shape[0] == 1 and s.number_bands != 1 else wx.shape[1]
        return cls(s.number_bands, s.nvband, s.ncouls, s.ngpown, s.nw, t(inp.aqsmtemp),
                   t(inp.aqsntemp), t(inp.I_eps_array), t(inp.wtilde_array), t(inp.vcoul),
                   t(inp.inv_igp_index), t(inp.indinv) if with_indinv else None, t(wx), stride)


def device_inputs(shape, seed: int = 20240607, device="cuda",
                  rows: tuple[int, int] | None = None) -> DeviceInputs:
    """Seeded workload generated directly in device memory (same bits as
    workload.make_inputs, without the host round trip).  rows = (r0, r1):
    only G' rows [r0, r1) of the G'-indexed arrays are made and held (one
    rank's share of a row-sharded state); ngpown is then r1 - r0."""
    from . import workload
    t = workload.make_inputs_device(shape, seed, device, rows=rows)
    stride = 0 if t["wx_array"].shape[0] == 1 and shape.number_bands != 1 else shape.nw
    ng = shape.ngpown if rows is None else rows[1] - rows[0]
    return DeviceInputs(shape.number_bands, shape.nvband, shape.ncouls, ng, shape.nw,
                        t["aqsmtemp"], t["aqsntemp"], t["I_eps_array"], t["wtilde_array"],
                        t["vcoul"], t["inv_igp_index"], t["indinv"], t["wx_array"], stride)


@dataclasses.dataclass
class SigmaResult:
    achtemp: "torch.Tensor"
    asxtemp: "torch.Tensor"
    acht_n1_loc: "torch.Tensor | None"
    achstemp: "torch.Tensor | None"


def problem_struct(d: DeviceInputs, precision: str, semantics: str, occ: float) -> capi.GppProblem:
    c128, f64, i32 = torch.complex128, torch.float64, torch.int32
    nb, nc, ng = d.number_bands, d.ncouls, d.ngpown
    p = capi.GppProblem()
    p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nw = nb, d.nvband, nc, ng, d.nw
    p.aqsmtemp = _ptr(d.aqsmtemp, c128, "aqsmtemp", nb * nc)
    p.aqsntemp = _ptr(d.aqsntemp, c128, "aqsntemp", nb * nc)
    p.I_eps_array = _ptr(d.I_eps_array, c128, "I_eps_array", ng * nc)
    p.wtilde_array = _ptr(d.wtilde_array, c128, "wtilde_array", ng * nc)
    p.vcoul = _ptr(d.vcoul, f64, "vcoul", nc)
    p.inv_igp_index = _ptr(d.inv_igp_index, i32, "inv_igp_index", ng)
    p.indinv = _ptr(d.indinv, i32, "indinv", nc) if d.indinv is not None else None
    p.wx_array = _ptr(d.wx_array, f64, "wx_array", d.nw if d.wx_stride == 0 else nb * d.wx_stride)
    p.wx_stride = d.wx_stride
    p.occ = float(occ)
    p.semantics = capi.SEMANTICS[semantics]
    p.precision = capi.PRECISION[precision]
    return p


def sigma(d: DeviceInputs, precision: str = "fp64", semantics: str = "complex_seq",
          occ: float = 1.0, acht_n1: bool = False, achstemp: bool = False,
          out: SigmaResult | None = None) -> SigmaResult:
    """achtemp/asxtemp (and optionally acht_n1_loc, achstemp) of the whole
    problem, computed on the current torch stream (asynchronous)."""
    lib = capi.load()
    dev = d.aqsmtemp.device
    if out is None:
        out = SigmaResult(torch.empty(d.nw, dtype=torch.complex128, device=dev),
                          torch.empty(d.nw, dtype=torch.complex128, device=dev),
                          torch.empty(d.number_bands, dtype=torch.complex128, device=dev) if acht_n1 else None,
                          torch.empty(1, dtype=torch.complex128, device=dev) if achstemp else None)
    p = problem_struct(d, precision, semantics, occ)
    o = capi.GppOutputs()
    o.achtemp = out.achtemp.data_ptr()
    o.asxtemp = out.asxtemp.data_ptr()
    o.acht_n1_loc = out.acht_n1_loc.data_ptr() if out.acht_n1_loc is not None else None
    o.achstemp = out.achstemp.data_ptr() if out.achstemp is not None else None
    capi.check(lib.gpp_sigma(C.byref(p), C.byref(o), _stream()), "gpp_sigma")
    return out


def autotune(d: DeviceInputs, max_bands: int = 64, semantics: str = "complex_seq") -> int:
    """Time the mixed kernel's pipeline variants on `d` (first `max_bands`
    unoccupied bands) and keep the fastest for this frequency chunk."""
    lib = capi.load()
    p = problem_struct(d, "mixed", semantics, 1.0)
    best = C.c_int(-1)
    capi.check(lib.gpp_autotune(C.byref(p), max_bands, _stream(), C.byref(best)), "gpp_autotune")
    return best.value


def set_variant(nw: int, variant: int) -> None:
    """Force a mixed-kernel pipeline variant for `nw` frequencies (-1: default)."""
    capi.check(capi.load().gpp_set_variant(nw, variant), "gpp_set_variant")


def variant_names() -> list[str]:
    lib = capi.load()
    return [lib.gpp_variant_name(i).decode() for i in range(lib.gpp_variant_count())]


def wait(timeout_ms: int = -1) -> None:
    """Synchronise the current stream and raise on device-side index faults."""
    capi.check(capi.load().gpp_wait(_stream(), timeout_ms), "gpp_wait")


class HostContext:
    """Device buffers + stream for the host-array path (gpp_sigma_host)."""

    def __init__(self):
        self._lib = capi.load()
        h = C.c_void_p()
        capi.check(self._lib.gpp_context_create(C.byref(h)), "gpp_context_create")
        self.handle = h

    def close(self):
        if self.handle:
            self._lib.gpp_context_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def sigma(self, arrays: dict, shape, precision="fp64", semantics="complex_seq", occ=1.0,
              acht_n1=False, achstemp=False) -> dict:
        """arrays: host numpy arrays (any memory; page-locked ones copy fastest)
        keyed like the reference's argument names; returns numpy outputs."""
        p = capi.GppProblem()
        p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nw = (
            shape.number_bands, shape.nvband, shape.ncouls, shape.ngpown, shape.nw)
        hp = lambda a: a.ctypes.data if a is not None else None
        p.aqsmtemp, p.aqsntemp = hp(arrays["aqsmtemp"]), hp(arrays["aqsntemp"])
        p.I_eps_array, p.wtilde_array = hp(arrays["I_eps_array"]), hp(arrays["wtilde_array"])
        p.vcoul, p.inv_igp_index = hp(arrays["vcoul"]), hp(arrays["inv_igp_index"])
        p.indinv = hp(arrays.get("indinv"))
        wx = arrays["wx_array"]
        p.wx_array = hp(wx)
        p.wx_stride = 0 if (wx.ndim == 1 or wx.shape[0] == 1) and shape.number_bands != 1 else wx.shape[-1]
        p.occ = float(occ)
        p.semantics = capi.SEMANTICS[semantics]
        p.precision = capi.PRECISION[precision]
        res = {"achtemp": np.zeros(shape.nw, np.complex128), "asxtemp": np.zeros(shape.nw, np.complex128)}
        o = capi.GppOutputs()
        o.achtemp, o.asxtemp = res["achtemp"].ctypes.data, res["asxtemp"].ctypes.data
        if acht_n1:
            res["acht_n1_loc"] = np.zeros(shape.number_bands, np.complex128)
            o.acht_n1_loc = res["acht_n1_loc"].ctypes.data
        if achstemp:
            res["achstemp"] = np.zeros(1, np.complex128)
            o.achstemp = res["achstemp"].ctypes.data
        capi.check(self._lib.gpp_sigma_host(self.handle, C.byref(p), C.byref(o)), "gpp_sigma_host")
        return res

    def last_trace(self) -> dict:
        """Timeline of the last sigma call (ms after its first copy): when the
        band arrays and each row piece landed, and when the kernels reached
        each piece."""
        n = C.c_int()
        buf = (C.c_float * (1 + 2 * 16))()
        capi.check(self._lib.gpp_context_last_trace(self.handle, buf, len(buf), C.byref(n)),
                   "gpp_context_last_trace")
        v = [round(buf[i], 2) for i in range(n.value)]
        return {"bands": v[0], "piece_landed": v[1::2], "piece_started": v[2::2]}

    def last_timing(self) -> dict:
        """Device-side milliseconds of the last sigma call: H2D copies,
        gpp_sigma, D2H copy (CUDA events on the context's stream)."""
        t = [C.c_float() for _ in range(3)]
        capi.check(self._lib.gpp_context_last_timing(self.handle, *[C.byref(x) for x in t]),
                   "gpp_context_last_timing")
        return {"h2d_ms": t[0].value, "compute_ms": t[1].value, "d2h_ms": t[2].value}

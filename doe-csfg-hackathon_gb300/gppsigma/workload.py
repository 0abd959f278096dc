"""Seeded synthetic GPP workloads (host side, numpy).

The reference mini-app synthesises its inputs in ``main`` (ramp values,
gppKerSeq.cpp:225-258).  The workloads here follow the same array shapes and
layouts with seeded random values:

* aqsmtemp / aqsntemp [number_bands][ncouls]: re, im ~ U(-0.5, 0.5)
* I_eps_array [ngpown][ncouls]: re, im ~ U(-0.5, 0.5)
* wtilde_array [ngpown][ncouls]: re ~ U(0.5, 2.0), im ~ U(-0.05, 0.05)
* vcoul [ncouls] ~ U(0.1, 1.0)
* inv_igp_index: ngpown distinct sorted G indices drawn from [0, ncouls)
* indinv: identity
* wx[n1][iw] = e_lk + dw*(iw+1) - e_n1, e_lk = 10, e_n1 ~ U(0, 20) per band,
  with the |wx| < to1 -> to1 clamp of gppKerSeq.cpp:257
* optionally a fraction of wtilde entries placed within 1e-4 of a wx value
  (near the plasmon pole)

Random numbers come from a counter-based SplitMix64 (Steele, Lea & Flood,
"Fast splittable pseudorandom number generators", 2014): value i of stream s
is mix(key_s + (i+1) * golden), so every array is reproducible bit for bit on
any host, independent of generation order or chunking.
"""
from __future__ import annotations

import dataclasses
import hashlib

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_TO1 = 1e-6
_CHUNK = 1 << 22

# Stream identifiers (one per array / component).
_S_AQSM_RE, _S_AQSM_IM, _S_AQSN_RE, _S_AQSN_IM = 1, 2, 3, 4
_S_IEPS_RE, _S_IEPS_IM, _S_WT_RE, _S_WT_IM = 5, 6, 7, 8
_S_VCOUL, _S_IGP, _S_EN1 = 9, 10, 11
_S_POLE_SEL, _S_POLE_BAND, _S_POLE_IW, _S_POLE_DRE, _S_POLE_DIM = 12, 13, 14, 15, 16
_S_STATE = 17


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def _key(seed: int, stream: int) -> np.uint64:
    with np.errstate(over="ignore"):
        z = np.array([(seed * 0x100000001B3 + stream * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF],
                     dtype=np.uint64)
        return _mix(_mix(z))[0]


def uniform(seed: int, stream: int, n: int, lo: float, hi: float, out: np.ndarray | None = None
            ) -> np.ndarray:
    """n doubles U(lo, hi) of stream `stream` (u = top 53 bits / 2^53)."""
    if out is None:
        out = np.empty(n, dtype=np.float64)
    key = _key(seed, stream)
    scale = hi - lo
    with np.errstate(over="ignore"):
        for s in range(0, n, _CHUNK):
            e = min(n, s + _CHUNK)
            ctr = np.arange(s + 1, e + 1, dtype=np.uint64)
            z = _mix(key + ctr * _GOLDEN)
            u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
            out[s:e] = lo + scale * u
    return out


def _complex(seed, s_re, s_im, rows, cols, lo_re, hi_re, lo_im, hi_im) -> np.ndarray:
    z = np.empty((rows, cols), dtype=np.complex128)
    v = z.view(np.float64).reshape(rows, cols, 2)
    n = rows * cols
    tmp = np.empty(n, dtype=np.float64)
    uniform(seed, s_re, n, lo_re, hi_re, tmp)
    v[..., 0] = tmp.reshape(rows, cols)
    uniform(seed, s_im, n, lo_im, hi_im, tmp)
    v[..., 1] = tmp.reshape(rows, cols)
    return z


@dataclasses.dataclass(frozen=True)
class Shape:
    number_bands: int
    nvband: int
    ncouls: int
    ngpown: int
    nw: int = 3
    dw: float = 1.0
    e_lk: float = 10.0
    near_pole: float = 0.0  # fraction of wtilde entries placed next to a wx value
    igp_overflow: int = 0   # trailing inv_igp_index entries set >= ncouls (clamp case)

    @property
    def terms(self) -> int:
        return self.number_bands * self.ngpown * self.ncouls * self.nw


# The reference's workload shapes (config 3, the batched set, is made by
# batched_shapes()).
CONFIGS: dict[str, Shape] = {
    # Small FP64 case the sequential CPU reference finishes in about a second.
    "small": Shape(512, 2, 2048, 128, 3),
    # The mini-app's production shape (FP64 kernel).
    "production": Shape(512, 2, 32768, 1638, 3),
    # Production shape with 1% of wtilde next to a wx value (mixed precision).
    "production_near_pole": Shape(512, 2, 32768, 1638, 3, near_pole=0.01),
    # Large single state with a 32-frequency sweep, dw = 0.25.
    "sweep32": Shape(2048, 8, 65536, 3277, 32, dw=0.25),
}


@dataclasses.dataclass
class Inputs:
    shape: Shape
    seed: int
    aqsmtemp: np.ndarray      # complex128 [nb][nc]
    aqsntemp: np.ndarray      # complex128 [nb][nc]
    I_eps_array: np.ndarray   # complex128 [ng][nc]
    wtilde_array: np.ndarray  # complex128 [ng][nc]
    vcoul: np.ndarray         # float64 [nc]
    inv_igp_index: np.ndarray # int32 [ng]
    indinv: np.ndarray        # int32 [nc]
    wx_array: np.ndarray      # float64 [nb][nw]

    def rows(self, r0: int, r1: int) -> "Inputs":
        """The same problem restricted to G' rows [r0, r1)."""
        sh = dataclasses.replace(self.shape, ngpown=r1 - r0)
        return dataclasses.replace(self, shape=sh, I_eps_array=self.I_eps_array[r0:r1],
                                   wtilde_array=self.wtilde_array[r0:r1],
                                   inv_igp_index=self.inv_igp_index[r0:r1])

    def digest(self) -> str:
        """sha256 over every input array's bytes (generator drift check)."""
        h = hashlib.sha256()
        for a in (self.aqsmtemp, self.aqsntemp, self.I_eps_array, self.wtilde_array, self.vcoul,
                  self.inv_igp_index, self.indinv, self.wx_array):
            h.update(np.ascontiguousarray(a).tobytes())
        return h.hexdigest()


def make_wx(shape: Shape, seed: int) -> np.ndarray:
    e_n1 = uniform(seed, _S_EN1, shape.number_bands, 0.0, 20.0)
    iw = np.arange(shape.nw, dtype=np.float64)
    wx = shape.e_lk + shape.dw * (iw[None, :] + 1.0) - e_n1[:, None]
    wx = np.where(np.abs(wx) < _TO1, _TO1, wx)
    return np.ascontiguousarray(wx)


def make_inputs(shape: Shape, seed: int = 20240607) -> Inputs:
    nb, nc, ng, nw = shape.number_bands, shape.ncouls, shape.ngpown, shape.nw
    if not (0 <= shape.nvband <= nb and nc > 0 and 0 <= ng <= nc and nw > 0):
        raise ValueError(f"bad shape {shape}")
    aqsm = _complex(seed, _S_AQSM_RE, _S_AQSM_IM, nb, nc, -0.5, 0.5, -0.5, 0.5)
    aqsn = _complex(seed, _S_AQSN_RE, _S_AQSN_IM, nb, nc, -0.5, 0.5, -0.5, 0.5)
    ieps = _complex(seed, _S_IEPS_RE, _S_IEPS_IM, ng, nc, -0.5, 0.5, -0.5, 0.5)
    wt = _complex(seed, _S_WT_RE, _S_WT_IM, ng, nc, 0.5, 2.0, -0.05, 0.05)
    vcoul = uniform(seed, _S_VCOUL, nc, 0.1, 1.0)
    keys = uniform(seed, _S_IGP, nc, 0.0, 1.0)
    igp = np.sort(np.argsort(keys, kind="stable")[:ng]).astype(np.int32)
    if shape.igp_overflow:
        k = min(shape.igp_overflow, ng)
        igp[ng - k:] = nc + np.arange(k, dtype=np.int32)
    wx = make_wx(shape, seed)
    if shape.near_pole > 0.0 and ng > 0:
        n = ng * nc
        sel = uniform(seed, _S_POLE_SEL, n, 0.0, 1.0) < shape.near_pole
        idx = np.flatnonzero(sel)
        band = np.minimum((uniform(seed, _S_POLE_BAND, n, 0.0, 1.0)[idx] * nb).astype(np.int64), nb - 1)
        iwk = np.minimum((uniform(seed, _S_POLE_IW, n, 0.0, 1.0)[idx] * nw).astype(np.int64), nw - 1)
        dre = uniform(seed, _S_POLE_DRE, n, -7e-5, 7e-5)[idx]
        dim = uniform(seed, _S_POLE_DIM, n, -7e-5, 7e-5)[idx]
        flat = wt.reshape(-1)
        flat[idx] = (wx[band, iwk] + dre) + 1j * dim
    indinv = np.arange(nc, dtype=np.int32)
    return Inputs(shape, seed, aqsm, aqsn, ieps, wt, vcoul, igp, indinv, wx)


def ramp_inputs(number_bands: int, nvband: int, ncouls: int, nodes_per_group: int) -> Inputs:
    """The reference's own ramp inputs (gppKerSeq.cpp:159-166, 225-258):
    ngpown = ncouls / nodes_per_group, band-independent wx = {3, 4, 5}."""
    nb, nc = number_bands, ncouls
    ng = nc // nodes_per_group
    nw = 3
    i_b = np.arange(nb, dtype=np.float64)[:, None]
    i_g = np.arange(ng, dtype=np.float64)[:, None]
    j = np.arange(nc, dtype=np.float64)[None, :]
    aq = (i_b + j) * 0.5
    aqs = aq + 1j * aq
    ge = (i_g + j) * 0.5
    gen = ge + 1j * ge
    igp = ((np.arange(ng, dtype=np.int64) + 1) * nc // ng).astype(np.int32)
    vcoul = np.arange(nc, dtype=np.float64)
    wx = np.array([10.0 - 6.0 + 1.0 * ((iw + 1) - 2) for iw in range(nw)], dtype=np.float64)
    wx = np.where(np.abs(wx) < _TO1, _TO1, wx)
    shape = Shape(nb, nvband, nc, ng, nw)
    return Inputs(shape, -1, aqs.copy(), aqs.copy(), gen.copy(), gen.copy(), vcoul, igp,
                  np.arange(nc, dtype=np.int32), wx[None, :].copy())


def batched_shapes(nstates: int = 64, seed: int = 20240607, scale: float = 1.0) -> list[Shape]:
    """Uneven quasiparticle states: number_bands ~ U{256..2048}, ncouls ~
    U{8192..65536}, ngpown = ncouls/20, nvband ~ U{2..8}, 3 frequencies.
    `scale` < 1 shrinks bands and ncouls proportionally (test sizes)."""
    u = uniform(seed, _S_STATE, 3 * nstates, 0.0, 1.0).reshape(nstates, 3)
    out = []
    for k in range(nstates):
        nb = 256 + int(u[k, 0] * (2048 - 256 + 1))
        nc = 8192 + int(u[k, 1] * (65536 - 8192 + 1))
        nv = 2 + int(u[k, 2] * 7)
        nb = max(nv, int(nb * scale))
        nc = max(20, int(nc * scale))
        out.append(Shape(nb, min(nv, nb), nc, nc // 20, 3))
    return out


# ---------------------------------------------------------------------------
# The same generator on a torch device (bit-identical to the numpy one): the
# SplitMix64 stream in int64 arithmetic (two's-complement wrap-around, logical
# shifts via masks), so large workloads are generated where they are used.

def _to_i64(u: int) -> int:
    u &= 0xFFFFFFFFFFFFFFFF
    return u - (1 << 64) if u >= (1 << 63) else u


def _lsr(z, k: int):
    import torch
    return torch.bitwise_and(torch.bitwise_right_shift(z, k), (1 << (64 - k)) - 1)


def _mix_t(z):
    z = torch_bitxor(z, _lsr(z, 30)) * _to_i64(int(_M1))
    z = torch_bitxor(z, _lsr(z, 27)) * _to_i64(int(_M2))
    return torch_bitxor(z, _lsr(z, 31))


def torch_bitxor(a, b):
    import torch
    return torch.bitwise_xor(a, b)


def uniform_t(seed: int, stream: int, n: int, lo: float, hi: float, device, out=None,
              offset: int = 0):
    """Device twin of uniform(): the same doubles, as a float64 tensor --
    values offset .. offset + n - 1 of the stream (the generator is
    counter-based, so any range comes out with the bits it has in the whole)."""
    import torch
    if out is None:
        out = torch.empty(n, dtype=torch.float64, device=device)
    key = _to_i64(int(_key(seed, stream)))
    golden = _to_i64(int(_GOLDEN))
    scale = hi - lo
    chunk = 1 << 26
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        ctr = torch.arange(offset + s + 1, offset + e + 1, dtype=torch.int64, device=device)
        z = _mix_t(ctr * golden + key)
        u = _lsr(z, 11).to(torch.float64) * (1.0 / 9007199254740992.0)
        out[s:e] = u * scale + lo
    return out


def _complex_t(seed, s_re, s_im, rows, cols, lo_re, hi_re, lo_im, hi_im, device, row0=0):
    """Rows row0 .. row0 + rows - 1 of a [*][cols] complex array."""
    import torch
    z = torch.empty((rows, cols), dtype=torch.complex128, device=device)
    v = torch.view_as_real(z).view(rows * cols, 2)
    n = rows * cols
    v[:, 0] = uniform_t(seed, s_re, n, lo_re, hi_re, device, offset=row0 * cols)
    v[:, 1] = uniform_t(seed, s_im, n, lo_im, hi_im, device, offset=row0 * cols)
    return z


def make_inputs_device(shape: Shape, seed: int = 20240607, device="cuda",
                       rows: tuple[int, int] | None = None) -> dict:
    """make_inputs() generated directly on `device` (torch tensors, same bits):
    keys aqsmtemp, aqsntemp, I_eps_array, wtilde_array, vcoul,
    inv_igp_index, indinv, wx_array.  With rows = (r0, r1) only the G' rows
    [r0, r1) of I_eps_array, wtilde_array and inv_igp_index are made (the
    share of one rank of a row-sharded state), with the bits those rows have
    in the whole state."""
    import torch
    nb, nc, ng, nw = shape.number_bands, shape.ncouls, shape.ngpown, shape.nw
    if not (0 <= shape.nvband <= nb and nc > 0 and 0 <= ng <= nc and nw > 0):
        raise ValueError(f"bad shape {shape}")
    r0, r1 = (0, ng) if rows is None else rows
    if not 0 <= r0 <= r1 <= ng:
        raise ValueError(f"bad row range {rows} for ngpown {ng}")
    nr = r1 - r0
    out = {
        "aqsmtemp": _complex_t(seed, _S_AQSM_RE, _S_AQSM_IM, nb, nc, -0.5, 0.5, -0.5, 0.5, device),
        "aqsntemp": _complex_t(seed, _S_AQSN_RE, _S_AQSN_IM, nb, nc, -0.5, 0.5, -0.5, 0.5, device),
        "I_eps_array": _complex_t(seed, _S_IEPS_RE, _S_IEPS_IM, nr, nc, -0.5, 0.5, -0.5, 0.5,
                                  device, row0=r0),
        "wtilde_array": _complex_t(seed, _S_WT_RE, _S_WT_IM, nr, nc, 0.5, 2.0, -0.05, 0.05,
                                   device, row0=r0),
        "vcoul": uniform_t(seed, _S_VCOUL, nc, 0.1, 1.0, device),
    }
    keys = uniform_t(seed, _S_IGP, nc, 0.0, 1.0, device)
    igp = torch.sort(torch.argsort(keys, stable=True)[:ng]).values.to(torch.int32)
    if shape.igp_overflow:
        k = min(shape.igp_overflow, ng)
        igp[ng - k:] = nc + torch.arange(k, dtype=torch.int32, device=device)
    out["inv_igp_index"] = igp[r0:r1].contiguous()
    wx = torch.from_numpy(make_wx(shape, seed)).to(device)
    if shape.near_pole > 0.0 and nr > 0:
        n, at = nr * nc, r0 * nc  # this range's elements of the [ng][nc] streams
        sel = uniform_t(seed, _S_POLE_SEL, n, 0.0, 1.0, device, offset=at) < shape.near_pole
        idx = torch.nonzero(sel).flatten()
        band = torch.clamp((uniform_t(seed, _S_POLE_BAND, n, 0.0, 1.0, device, offset=at)[idx] * nb).to(torch.int64), max=nb - 1)
        iwk = torch.clamp((uniform_t(seed, _S_POLE_IW, n, 0.0, 1.0, device, offset=at)[idx] * nw).to(torch.int64), max=nw - 1)
        dre = uniform_t(seed, _S_POLE_DRE, n, -7e-5, 7e-5, device, offset=at)[idx]
        dim = uniform_t(seed, _S_POLE_DIM, n, -7e-5, 7e-5, device, offset=at)[idx]
        flat = torch.view_as_real(out["wtilde_array"]).view(-1, 2)
        flat[idx, 0] = wx[band, iwk] + dre
        flat[idx, 1] = dim
    out["indinv"] = torch.arange(nc, dtype=torch.int32, device=device)
    out["wx_array"] = wx.contiguous()
    return out

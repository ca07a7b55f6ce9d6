"""Device-side generator of the seeded synthetic systems, for served request streams.

The same construction as ``synth.make_system`` (Kramers-paired time-reversal-symmetric
Hermitian factors B^L, L = nmo, (pq|rs) = sum_L B^L_pq B^L_rs, canonical MDCINTNEW
representatives by the TYPE1-4 filter of create_newmdcint.F90:286-320, the orbits the path
never reads omitted), with the random numbers drawn by torch's generator on the target device
and the block contractions run there, so that a stream of hundreds of requests of up to
~10^8 records each is produced in seconds and its records stay in HBM (the ``rec_on_device``
input of dcg_set_system).  The record index set is identical to ``synth.make_system``'s for
the same sizes; the values differ (another random stream), and with ``gemm_dtype =
torch.complex64`` the integrals are FP32-representable numbers held in FP64.
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import List, Optional

import numpy as np
import torch

from . import api
from .synth import SynthConfig, _space_ranges, _used_pattern

__all__ = ["DeviceSystem", "make_system_device", "canonical_mask_t", "stream_configs"]

CHUNK_ELEMENTS = 1 << 27   # dense integral elements contracted at once (first-index chunks)


@dataclasses.dataclass
class DeviceSystem:
    cfg: SynthConfig
    nmo: int
    h: np.ndarray                  # (nmo, nmo) complex128, host
    ecore: float
    rec_idx: torch.Tensor          # (nrec, 4) int32, 1-based, on the device
    rec_re: torch.Tensor           # (nrec,) float64
    rec_im: Optional[torch.Tensor]  # (nrec,) float64, None when realonly
    B: Optional[torch.Tensor] = None   # (L, nmo, nmo) factors when kept

    @property
    def nrec(self) -> int:
        return int(self.rec_re.numel())

    @property
    def record_bytes(self) -> int:
        return int(self.rec_idx.numel() * 4 + self.rec_re.numel() * 8 +
                   (self.rec_im.numel() * 8 if self.rec_im is not None else 0))

    def system_input(self, selectroot: int = 1, ras=(0, 0, 0), ras1_max_hole: int = 0,
                     ras3_max_elec: int = 0) -> api.SystemInput:
        """The dcg_system fields with empty host records (the records are on the device); a
        RAS partition of the active spinors is optional."""
        c = self.cfg
        return api.SystemInput(ninact=c.ninact, nact=c.nact, nsec=c.nsec, nelec=c.nelec, nmo=self.nmo,
                               nsymrpa=1, multb=np.array([[2, 1], [1, 2]]), irpamo=np.ones(self.nmo, np.int64),
                               h=self.h, ecore=self.ecore, rec_idx=np.zeros((0, 4), np.int32),
                               rec_val=np.zeros(0, np.complex128), realonly=c.realonly, selectroot=selectroot,
                               eshift=c.eshift, ras=tuple(ras), ras1_max_hole=ras1_max_hole,
                               ras3_max_elec=ras3_max_elec)

    def buffers(self, selectroot: int = 1, **ras) -> api.HostBuffers:
        """HostBuffers whose dcg_system points at the device records."""
        b = api.HostBuffers(self.system_input(selectroot, **ras))
        b.use_device_records(self.rec_idx.data_ptr(), self.rec_re.data_ptr(),
                             self.rec_im.data_ptr() if self.rec_im is not None else 0)
        b.struct.nrec = self.nrec
        b.device_system = self   # keeps the device tensors alive with the buffers
        return b


def _normal(gen: torch.Generator, shape, scale: float, device) -> torch.Tensor:
    return torch.randn(shape, generator=gen, device=device, dtype=torch.float64) * scale


def _tr_hermitian_batch(gen, nb: int, npair: int, scale: float, diag: Optional[torch.Tensor], realonly: bool,
                        device) -> torch.Tensor:
    """nb random Hermitian time-reversal-symmetric matrices in the Kramers-paired basis: pair
    block (p, q) = [[a, b], [-conj(b), conj(a)]] with a Hermitian, b antisymmetric, real
    diagonal of a (``diag``, or N(0, scale^2))."""
    def cplx():
        re = _normal(gen, (nb, npair, npair), scale, device)
        im = _normal(gen, (nb, npair, npair), scale, device)
        return torch.complex(re, torch.zeros_like(im) if realonly else im)

    a = torch.triu(cplx(), 1)
    a = a + a.conj().transpose(1, 2)
    b = torch.triu(cplx(), 1)
    b = b - b.transpose(1, 2)
    d = diag if diag is not None else _normal(gen, (nb, npair), scale, device)
    a = a + torch.diag_embed(d.to(torch.complex128))
    n = 2 * npair
    M = torch.zeros((nb, n, n), dtype=torch.complex128, device=device)
    M[:, 0::2, 0::2] = a
    M[:, 0::2, 1::2] = b
    M[:, 1::2, 0::2] = -b.conj()
    M[:, 1::2, 1::2] = a.conj()
    return M


def canonical_mask_t(p: torch.Tensor, q: torch.Tensor, r: torch.Tensor, s: torch.Tensor) -> torch.Tensor:
    """Torch form of ``synth._canonical_mask``: the record (p, q, r, s) (0-based, broadcast) is
    the one create_newmdcint writes when its Kramers partners pass the TYPE1-4 filter."""
    i, j, k, l = ((x ^ 1) + 1 for x in (p, q, r, s))

    def kr(x):
        return torch.where(x % 2 == 1, 1, -1) * (x // 2 + x % 2)

    ik, jk, kk_, lk = kr(i), kr(j), kr(k), kr(l)
    ii, jj, kk, ll = ik.abs(), jk.abs(), kk_.abs(), lk.abs()
    t1 = (ik > 0) & (jk > 0) & (kk_ > 0) & (lk > 0)
    t2 = (ik > 0) & (jk < 0) & (kk_ > 0) & (lk < 0)
    t3 = (ik > 0) & (jk < 0) & (kk_ < 0) & (lk > 0)
    t4 = (ik > 0) & (jk < 0) & (kk_ < 0) & (lk < 0)
    c1 = ((ii <= jj) & (kk <= ll) & ((ii < kk) | ((ii == kk) & (jj <= ll)))) | \
         ((ii <= jj) & (ll <= kk) & ((ii < ll) | ((ii == ll) & (jj <= kk))))
    c23 = (ii <= jj) & (kk <= ll) & ((ii < kk) | ((ii == kk) & (jj <= ll)))
    return (t1 & c1) | (t2 & c23) | (t3 & c23) | (t4 & (ii <= jj))


def make_system_device(cfg: SynthConfig, device="cuda", gemm_dtype: Optional[torch.dtype] = None,
                       keep_factors: bool = False) -> DeviceSystem:
    """Build the synthetic system of ``cfg`` on ``device`` (deterministic in ``cfg.seed`` for a
    given device type).  ``gemm_dtype`` is the dtype of the factor contraction (default
    complex64 on CUDA, complex128 elsewhere)."""
    ni, na, ns = cfg.ninact, cfg.nact, cfg.nsec
    for v, nm in ((ni, "ninact"), (na, "nact"), (ns, "nsec")):
        if v % 2:
            raise ValueError(f"{nm} must be even (Kramers pairs)")
    device = torch.device(device)
    if gemm_dtype is None:
        gemm_dtype = torch.complex64 if device.type == "cuda" else torch.complex128
    nmo = ni + na + ns
    npair = nmo // 2
    gen = torch.Generator(device=device)
    gen.manual_seed(int(cfg.seed))

    def uni(n, lo, hi):
        return torch.sort(torch.rand(n, generator=gen, device=device, dtype=torch.float64) * (hi - lo) + lo).values

    e_pair = torch.cat([uni(ni // 2, -20.0, -1.0), uni(na // 2, -0.5, 0.2), uni(ns // 2, 0.3, 50.0)])
    h = _tr_hermitian_batch(gen, 1, npair, 0.01, e_pair[None], cfg.realonly, device)[0]
    L = nmo
    B = _tr_hermitian_batch(gen, L, npair, 0.05 / np.sqrt(L), None, cfg.realonly, device)
    ecore = float(torch.rand(1, generator=gen, device=device, dtype=torch.float64).item() * 25.0 + 5.0)
    Bg = B.to(gemm_dtype)
    if not keep_factors:
        del B
        B = None
    ranges = _space_ranges(cfg)
    idx_out: List[torch.Tensor] = []
    val_out: List[torch.Tensor] = []
    for sp in itertools.product((1, 2, 3), repeat=4):
        if not _used_pattern(sp):
            continue
        r = [ranges[x] for x in sp]
        if any(b - a == 0 for a, b in r):
            continue
        Q, R, S = (torch.arange(a, b, device=device) for a, b in r[1:])
        Brs = Bg[:, r[2][0]:r[2][1], r[3][0]:r[3][1]].reshape(L, -1)
        # first-index chunks bound the dense block held at once to ~2^27 elements; the
        # record order stays the C order of the whole block
        step = max(1, CHUNK_ELEMENTS // max(1, len(Q) * len(R) * len(S)))
        for p0 in range(r[0][0], r[0][1], step):
            p1 = min(p0 + step, r[0][1])
            P = torch.arange(p0, p1, device=device)
            mask = canonical_mask_t(P[:, None, None, None], Q[None, :, None, None], R[None, None, :, None],
                                    S[None, None, None, :])
            sel = torch.nonzero(mask.expand(len(P), len(Q), len(R), len(S)))
            if sel.numel() == 0:
                continue
            Bpq = Bg[:, p0:p1, r[1][0]:r[1][1]].reshape(L, -1)
            blk = (Bpq.transpose(0, 1) @ Brs).reshape(len(P), len(Q), len(R), len(S))
            vals = blk[sel[:, 0], sel[:, 1], sel[:, 2], sel[:, 3]].to(torch.complex128)
            del blk
            idx = torch.stack([P[sel[:, 0]], Q[sel[:, 1]], R[sel[:, 2]], S[sel[:, 3]]], dim=1) + 1
            idx_out.append(idx.to(torch.int32))
            val_out.append(vals)
            del sel
    rec_idx = torch.cat(idx_out).contiguous() if idx_out else torch.zeros((0, 4), dtype=torch.int32, device=device)
    val = torch.cat(val_out) if val_out else torch.zeros(0, dtype=torch.complex128, device=device)
    rec_re = val.real.contiguous()
    rec_im = None if cfg.realonly else val.imag.contiguous()
    del val, Bg
    return DeviceSystem(cfg=cfg, nmo=nmo, h=h.cpu().numpy(), ecore=ecore, rec_idx=rec_idx, rec_re=rec_re,
                        rec_im=rec_im, B=B)


def stream_configs(n: int, seed: int = 0, nact_choices=(4, 6, 8, 10, 12), ninact_range=(4, 24),
                   nsec_range=(60, 400)) -> List[SynthConfig]:
    """Sizes of a served stream: per request an independent seed, active spinors uniform in
    ``nact_choices`` (half filled), inactive and secondary uniform over the even numbers of
    their ranges."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        na = int(rng.choice(nact_choices))
        ni = 2 * int(rng.integers(ninact_range[0] // 2, ninact_range[1] // 2 + 1))
        ns = 2 * int(rng.integers(nsec_range[0] // 2, nsec_range[1] // 2 + 1))
        out.append(SynthConfig(ni, na, ns, na // 2, seed=int(rng.integers(0, 2**31 - 1)),
                               name=f"req{k}_{ni}_{na}_{ns}"))
    return out

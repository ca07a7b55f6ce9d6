"""Seeded synthetic Kramers-paired systems for tests and benchmarks.

The workloads are the CASCI/CASPT2 configurations the project measures: complex128
Kramers-paired spinors without point-group symmetry (nsymrpa = 1), orbital energies drawn
uniformly per class (inactive [-20,-1], active [-0.5,0.2], secondary [0.3,50] Eh),
Hermitian one-electron integrals with N(0, 0.01^2) off-diagonals, and two-electron
integrals from a Kramers-symmetric density-fitting form

    (pq|rs) = sum_L B^L_pq B^L_rs,   B^L Hermitian and time-reversal symmetric,
    B^L entries ~ N(0, 0.05^2 / L),  L = nmo

(equivalently sum_L B^L_pq conj(B^L_sr)), which has the full 8-fold permutational and
Kramers symmetry of relativistic spinor integrals and a positive semidefinite Coulomb metric.

Time-reversal convention (the one the reference readers assume,
``module_2integrals.F90:395-434``, ``takekr.F90:17-144``): spinors 2m-1 (unbarred) and
2m (barred) form Kramers pair m, and a time-reversal-symmetric operator satisfies
O[x~, y~] = (-1)^(x+y) conj(O[x, y]) with x~ the partner of x (1-based indices).

Records are produced in MDCINTNEW form: one canonical representative per symmetry orbit,
chosen with the reference's TYPE1-4 filter (``create_newmdcint.F90:286-320``) applied to the
Kramers partners, exactly as DIRAC's MDCINT would yield after ``create_newmdcint``.
Orbits the hot path never reads ((ss|ss), (ss|pq) with p, q in different spaces) are
omitted; the readers skip them (``module_2integrals.F90:392``,
``divide_2_elec_integral_into_subspaces.F90:111-116``).
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import Dict, Optional, Tuple

import numpy as np

__all__ = ["SynthConfig", "SynthSystem", "make_system", "CONFIGS", "write_case_files"]


@dataclasses.dataclass(frozen=True)
class SynthConfig:
    ninact: int
    nact: int
    nsec: int
    nelec: int
    realonly: bool = False
    seed: int = 0
    eshift: float = 0.0
    name: str = ""


CONFIGS = {
    # Plain CASCI/CASPT2, complex128, no symmetry: 8 inactive, 6 active (4 e), 40 secondary
    "cas_8_6_40": SynthConfig(8, 6, 40, 4, name="cas_8_6_40"),
    # transformation-dominated case: 20 inactive, 12 active (6 e), 300 secondary
    "cas_20_12_300": SynthConfig(20, 12, 300, 6, name="cas_20_12_300"),
    # large single solve: 40 inactive, 14 active (8 e), 800 secondary
    "cas_40_14_800": SynthConfig(40, 14, 800, 8, name="cas_40_14_800"),
    # the same active space and inactive count with 160 secondary spinors: every active-space
    # structure of the large solve (3003 determinants, 2744-dimensional A and C blocks, Gram
    # factors of 2002 rows) at a size the CPU oracle finishes in minutes
    "cas_40_14_160": SynthConfig(40, 14, 160, 8, name="cas_40_14_160"),
}


@dataclasses.dataclass
class SynthSystem:
    cfg: SynthConfig
    nmo: int
    h: np.ndarray            # (nmo, nmo) complex, CAS order
    mo_energy: np.ndarray    # (nmo,)
    ecore: float
    rec_idx: np.ndarray      # (n, 4) int32 1-based MDCINTNEW indices
    rec_val: np.ndarray      # (n,) complex128
    B: Optional[np.ndarray] = None   # (L, nmo, nmo) factors (kept for small systems)

    @property
    def irpamo(self) -> np.ndarray:
        return np.ones(self.nmo, dtype=np.int64)

    @property
    def multb(self) -> np.ndarray:
        return np.array([[2, 1], [1, 2]], dtype=np.int64)

    def dense_g(self) -> np.ndarray:
        """Full (pq|rs) tensor (small systems only)."""
        return np.einsum("Lpq,Lrs->pqrs", self.B, self.B, optimize=True)


def _tr_hermitian(rng: np.random.Generator, npair: int, scale: float, diag: Optional[np.ndarray],
                  realonly: bool) -> np.ndarray:
    """Random Hermitian, time-reversal-symmetric matrix in the Kramers-paired basis.

    Pair block (rows p,p~; cols q,q~) = [[a, b], [-conj(b), conj(a)]]; diagonal blocks have
    real a and b = 0."""
    n = 2 * npair
    a = rng.normal(0.0, scale, (npair, npair)) + 1j * rng.normal(0.0, scale, (npair, npair))
    b = rng.normal(0.0, scale, (npair, npair)) + 1j * rng.normal(0.0, scale, (npair, npair))
    if realonly:
        a = a.real + 0j
        b = b.real + 0j
    # Hermitian in the pair index: a(q,p) = conj(a(p,q)), b(q,p) = -b(p,q)^T-consistent
    a = np.triu(a, 1)
    a = a + np.conj(a).T
    b = np.triu(b, 1)
    b = b - b.T            # [[a,b],[-b*,a*]] Hermitian requires b(q,p) = -b(p,q)
    d = diag if diag is not None else rng.normal(0.0, scale, npair)
    a = a + np.diag(d)
    M = np.zeros((n, n), dtype=np.complex128)
    M[0::2, 0::2] = a
    M[0::2, 1::2] = b
    M[1::2, 0::2] = -np.conj(b)
    M[1::2, 1::2] = np.conj(a)
    return M


def _partner0(x: np.ndarray) -> np.ndarray:
    """0-based Kramers partner."""
    return x ^ 1


def _canonical_mask(p: np.ndarray, q: np.ndarray, r: np.ndarray, s: np.ndarray) -> np.ndarray:
    """True where the MDCINTNEW record (p,q,r,s) (0-based) is the representative that
    ``create_newmdcint`` writes: its Kramers partners (i,j,k,l) pass the TYPE1-4 filter
    (create_newmdcint.F90:296-320)."""
    i, j, k, l = (_partner0(x) + 1 for x in (p, q, r, s))     # 1-based DIRAC-side indices

    def kr(x):
        return np.where(x % 2 == 1, 1, -1) * (x // 2 + x % 2)

    ik, jk, kk_, lk = kr(i), kr(j), kr(k), kr(l)
    ii, jj, kk, ll = np.abs(ik), np.abs(jk), np.abs(kk_), np.abs(lk)
    t1 = (ik > 0) & (jk > 0) & (kk_ > 0) & (lk > 0)
    t2 = (ik > 0) & (jk < 0) & (kk_ > 0) & (lk < 0)
    t3 = (ik > 0) & (jk < 0) & (kk_ < 0) & (lk > 0)
    t4 = (ik > 0) & (jk < 0) & (kk_ < 0) & (lk < 0)
    c1 = ((ii <= jj) & (kk <= ll) & ((ii < kk) | ((ii == kk) & (jj <= ll)))) | \
         ((ii <= jj) & (ll <= kk) & ((ii < ll) | ((ii == ll) & (jj <= kk))))
    c23 = (ii <= jj) & (kk <= ll) & ((ii < kk) | ((ii == kk) & (jj <= ll)))
    return (t1 & c1) | (t2 & c23) | (t3 & c23) | (t4 & (ii <= jj))


def _space_ranges(cfg: SynthConfig):
    ni, na, ns = cfg.ninact, cfg.nact, cfg.nsec
    return {1: (0, ni), 2: (ni, ni + na), 3: (ni + na, ni + na + ns)}


def _used_pattern(sp: Tuple[int, int, int, int]) -> bool:
    """Space patterns (of one orbit member) whose orbit the hot path reads."""
    a, b, c, d = sp
    p1 = tuple(sorted((a, b)))
    p2 = tuple(sorted((c, d)))
    if p1 == (3, 3) and p2 == (3, 3):
        return False
    if p1 == (3, 3):
        return p2 in ((1, 1), (2, 2))
    if p2 == (3, 3):
        return p1 in ((1, 1), (2, 2))
    return True


def make_system(cfg: SynthConfig, keep_factors: Optional[bool] = None) -> SynthSystem:
    """Build the seeded synthetic system of ``cfg`` (deterministic in ``cfg.seed``)."""
    ni, na, ns = cfg.ninact, cfg.nact, cfg.nsec
    for v, nm in ((ni, "ninact"), (na, "nact"), (ns, "nsec")):
        if v % 2:
            raise ValueError(f"{nm} must be even (Kramers pairs)")
    nmo = ni + na + ns
    npair = nmo // 2
    rng = np.random.default_rng(cfg.seed)
    e_in = np.sort(rng.uniform(-20.0, -1.0, ni // 2))
    e_ac = np.sort(rng.uniform(-0.5, 0.2, na // 2))
    e_se = np.sort(rng.uniform(0.3, 50.0, ns // 2))
    e_pair = np.concatenate([e_in, e_ac, e_se])
    h = _tr_hermitian(rng, npair, 0.01, e_pair, cfg.realonly)
    mo_energy = np.repeat(e_pair, 2)
    L = nmo
    B = np.stack([_tr_hermitian(rng, npair, 0.05 / np.sqrt(L), None, cfg.realonly) for _ in range(L)])
    ecore = float(rng.uniform(5.0, 30.0))
    ranges = _space_ranges(cfg)
    idx_out, val_out = [], []
    # enumerate blocks of space patterns; canonical members are unique across blocks
    for sp in itertools.product((1, 2, 3), repeat=4):
        if not _used_pattern(sp):
            continue
        r = [ranges[x] for x in sp]
        if any(b - a == 0 for a, b in r):
            continue
        P = np.arange(r[0][0], r[0][1])
        Q = np.arange(r[1][0], r[1][1])
        R = np.arange(r[2][0], r[2][1])
        S = np.arange(r[3][0], r[3][1])
        # dense block by one GEMM over the fitting index, then the canonical entries
        Bpq = B[:, r[0][0]:r[0][1], r[1][0]:r[1][1]].reshape(L, -1)
        Brs = B[:, r[2][0]:r[2][1], r[3][0]:r[3][1]].reshape(L, -1)
        blk = (Bpq.T @ Brs).reshape(len(P), len(Q), len(R), len(S))
        pp, qq, rr, ss = np.meshgrid(P, Q, R, S, indexing="ij", sparse=True)
        mask = np.broadcast_to(_canonical_mask(pp, qq, rr, ss), blk.shape)
        if not np.any(mask):
            continue
        sel = np.nonzero(mask)
        pi, qi, ri, si = P[sel[0]], Q[sel[1]], R[sel[2]], S[sel[3]]
        vals = blk[sel]
        del blk
        idx_out.append(np.stack([pi, qi, ri, si], axis=1).astype(np.int32) + 1)
        val_out.append(vals)
    rec_idx = np.concatenate(idx_out) if idx_out else np.zeros((0, 4), np.int32)
    rec_val = np.concatenate(val_out) if val_out else np.zeros(0, np.complex128)
    if cfg.realonly:
        rec_val = rec_val.real + 0j
    if keep_factors is None:
        keep_factors = nmo <= 80
    return SynthSystem(cfg=cfg, nmo=nmo, h=h, mo_energy=mo_energy, ecore=ecore,
                       rec_idx=rec_idx, rec_val=rec_val, B=B if keep_factors else None)


# --------------------------------------------------------------------------------------
# DIRAC-format files for a synthetic system (small systems: exercises the readers)
# --------------------------------------------------------------------------------------
def write_mrconee(path: str, nmo: int, ecore: float, h: np.ndarray, mo_energy: np.ndarray, diracver: int = 21,
                  nsymrpa: int = 1, multb: Optional[np.ndarray] = None, irpamo: Optional[np.ndarray] = None) -> None:
    """MRCONEE in the 64-bit DIRAC layout (read_mrconee.F90:226-600) with the spinors already
    in energy (CAS) order: records NMO/ECORE, irreps, MULTB (2n x 2n, [i0-1, j0-1] =
    MULTB(i0, j0)), (IRPMO, IRPAMO, energy) and the one-electron integrals."""
    import struct
    from .dirac_io import write_fortran_records
    i8 = lambda *xs: struct.pack("<" + "q" * len(xs), *xs)
    n2 = 2 * nsymrpa
    mb = np.array([[2, 1], [1, 2]], np.int64) if multb is None else np.asarray(multb, np.int64)
    irp = np.ones(nmo, np.int64) if irpamo is None else np.asarray(irpamo, np.int64)
    r1 = i8(nmo, 0) + struct.pack("<d", ecore) + i8(1, 2, 0, nmo) + struct.pack("<d", 0.0)
    r2 = i8(n2) + b"".join(f"{k + 1:>4d}A         ".encode()[:14] for k in range(n2))
    r3 = i8(nsymrpa) + b"".join(f"{k + 1:>4d}"[-4:].encode() for k in range(n2))
    r4 = i8(*[int(x) for x in mb.T.reshape(-1)])          # Fortran column-major
    r5 = b"".join(i8(int(irp[k]), int(irp[k])) + struct.pack("<d", float(mo_energy[k])) for k in range(nmo))
    onei = -h.imag if diracver >= 21 else h.imag
    r6 = np.stack([h.real, onei], axis=2).astype("<f8").tobytes()   # ((ONER(i,j),ONEI(i,j),j),i)
    write_fortran_records(path, [r1, r2, r3, r4, r5, r6])


def write_mdcint(path: str, nmo: int, rec_idx: np.ndarray, rec_val: np.ndarray, realonly: bool) -> None:
    """MDCINT (64-bit, scheme 6) holding the given MDCINTNEW records: header with the Kramers
    table, one record per signed Kramers index pair of the DIRAC-side (i, j), values conjugated
    as create_newmdcint undoes (create_newmdcint.F90:171-177), end record."""
    import struct
    from .dirac_io import write_fortran_records
    i8 = lambda *xs: struct.pack("<" + "q" * len(xs), *xs)
    npair = nmo // 2
    hdr = b" 01Jan26  " + b"00:00:00" + i8(npair) + b"".join(i8(2 * m - 1, 2 * m) for m in range(1, npair + 1))
    p = np.asarray(rec_idx).astype(np.int64) - 1
    dirac = (p ^ 1) + 1                                           # DIRAC-side 1-based spinors
    signed = np.where(dirac % 2 == 1, 1, -1) * ((dirac + 1) // 2)
    w = np.conj(np.asarray(rec_val))
    order = np.lexsort((signed[:, 1], signed[:, 0]))
    signed, w = signed[order], w[order]
    recs = [hdr]
    keys = signed[:, 0] * (npair + 1) * 4 + signed[:, 1]
    if len(keys):
        starts = np.flatnonzero(np.r_[True, keys[1:] != keys[:-1]])
        ends = np.r_[starts[1:], len(keys)]
        for a, b in zip(starts, ends):
            nz = b - a
            kl = signed[a:b, 2:4].astype("<i8").tobytes()
            if realonly:
                vv = w[a:b].real.astype("<f8").tobytes()
            else:
                vv = np.stack([w[a:b].real, w[a:b].imag], axis=1).astype("<f8").tobytes()
            recs.append(i8(int(signed[a, 0]), int(signed[a, 1]), int(nz)) + kl + vv)
    recs.append(i8(0, 0, 0))
    write_fortran_records(path, recs)


def write_case_files(sysm: SynthSystem, directory: str, diracver: int = 21) -> None:
    """Write active.inp, MRCONEE and MDCINT (64-bit DIRAC layout, scheme 6) such that the
    reference readers reproduce ``sysm`` exactly."""
    import os
    from .dirac_io import ActiveInput
    cfg = sysm.cfg
    os.makedirs(directory, exist_ok=True)
    inp = ActiveInput(ninact=cfg.ninact, nact=cfg.nact, nsec=cfg.nsec, nelec=cfg.nelec,
                      ciroots=[(1, 1)], eshift=cfg.eshift, diracver=diracver, scheme=6)
    open(os.path.join(directory, "active.inp"), "w").write(inp.to_text())
    write_mrconee(os.path.join(directory, "MRCONEE"), sysm.nmo, sysm.ecore, sysm.h, sysm.mo_energy, diracver)
    write_mdcint(os.path.join(directory, "MDCINT"), sysm.nmo, sysm.rec_idx, sysm.rec_val, cfg.realonly)

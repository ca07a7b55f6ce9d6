"""CPU oracle for the DIRAC-CASPT2 hot path (test infrastructure only).

This module is the CHECKER for the GPU library: a numpy restatement of the reference's
FP64 Fortran algorithm for CASCI, the CASCI-state Fock build and diagonalisation, the CI
rotation into the Fock-diagonal spinor basis, the 4-index transformation and the eight
subspace solvers A-H.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import it; the product path never does.

Parity of this oracle is pinned against the reference's own golden outputs
(``test/dev/*/reference.*.out``) by ``tests/test_oracle_golden.py``.

Every function cites the reference file and lines (paths inside the reference project)
whose behaviour it restates.  Index convention here: 0-based global CAS-order spinors
``0..nmo-1`` (inactive, active, secondary); active spinor ``t`` <-> bit ``t`` of a
determinant bit string.

Two evaluation modes for the ``dimN_density`` elements:
  * ``literal``: the determinant loop of ``density_matrix.F90:3-247`` element by element
    (small cases only);
  * ``rdm``: the same expectation values precomputed as dense tensors through the full
    N-electron space (identical numbers to rounding; validated against ``literal``).
"""
from __future__ import annotations

import dataclasses
import functools
import math
from typing import Dict, List, Optional, Tuple

import numpy as np

SMAT_LIN_DEP_THRESHOLD = 1.0e-8     # module_global_variables.F90:181
BMAT_NO_CUTOFF = 0.0                # module_global_variables.F90:182
INTRA_CUTOFF = 1.0e-15              # module_intra.F90:85 (write cutoff of transformed classes)
EFFH_C_SKIP = 1.0e-10               # solve_C_subspace.F90 vCmat: |effh(a,p)| < 1e-10 skipped

SUBSPACES = "ABCDEFGH"


# ======================================================================================
# System description
# ======================================================================================
@dataclasses.dataclass
class System:
    """Everything the hot path consumes, in CAS order (0-based)."""
    ninact: int
    nact: int
    nsec: int
    nelec: int
    nmo: int
    nsymrpa: int
    multb: np.ndarray          # (2n,2n) 1-based values, Fortran (i0,j0) at [i0-1, j0-1]
    irpamo: np.ndarray         # (nmo,) 1-based irreps
    h: np.ndarray              # (nmo, nmo) complex
    ecore: float
    rec_idx: np.ndarray        # (n,4) 1-based MDCINTNEW indices
    rec_val: np.ndarray        # (n,) complex
    realonly: bool
    totsym: int = 1
    selectroot: int = 1
    eshift: float = 0.0
    ras1: Tuple[int, ...] = ()
    ras2: Tuple[int, ...] = ()
    ras3: Tuple[int, ...] = ()
    ras1_max_hole: int = 0
    ras3_max_elec: int = 0
    min_hole_ras1: int = 0
    min_elec_ras3: int = 0

    @property
    def nmoc(self) -> int:
        return self.ninact + self.nact

    @functools.cached_property
    def _space_lut(self) -> np.ndarray:
        n = max(self.nmo, self.ninact + self.nact + self.nsec)
        lut = np.full(n + 1, 4, dtype=np.int8)
        lut[:self.ninact + self.nact + self.nsec] = 3
        lut[:self.ninact + self.nact] = 2
        lut[:self.ninact] = 1
        return lut

    def space_of(self, g: np.ndarray) -> np.ndarray:
        """1 inactive, 2 active, 3 secondary, 4 beyond (read_mrconee.F90:311-315)."""
        return self._space_lut[np.asarray(g)]

    # multiplication tables (read_mrconee.F90:368-453)
    @functools.cached_property
    def multb_s(self):
        n = self.nsymrpa
        return self.multb[n:2 * n, n:2 * n] - n

    @functools.cached_property
    def multb2(self):
        n2 = 2 * self.nsymrpa
        m2 = np.zeros((n2, n2), dtype=np.int64)
        for i0 in range(n2):
            for j0 in range(n2):
                m2[i0, self.multb[i0, j0] - 1] = j0 + 1
        return m2

    @functools.cached_property
    def multb_d(self):
        n = self.nsymrpa
        return self.multb2[0:n, 0:n] - n

    @functools.cached_property
    def multb_ds(self):
        n = self.nsymrpa
        return np.ascontiguousarray(self.multb[n:2 * n, 0:n].T)


def system_from_files(directory: str, totsym: Optional[int] = None, selectroot: Optional[int] = None) -> System:
    """Read active.inp, MRCONEE and MDCINT* of a reference-style case directory."""
    import os
    from dirac_caspt2_gb300 import dirac_io
    inp = dirac_io.read_active_inp(os.path.join(directory, "active.inp"))
    mrc = dirac_io.read_mrconee(os.path.join(directory, "MRCONEE"), inp)
    new = dirac_io.read_mdcint_new(directory, mrc, inp)
    ts, sr = inp.ciroots[0]
    return System(ninact=inp.ninact, nact=inp.nact, nsec=inp.nsec, nelec=inp.nelec, nmo=mrc.nmo,
                  nsymrpa=mrc.nsymrpa, multb=mrc.multb, irpamo=mrc.irpamo, h=mrc.h, ecore=mrc.ecore,
                  rec_idx=new.idx, rec_val=new.val, realonly=new.realonly,
                  totsym=totsym if totsym is not None else ts,
                  selectroot=selectroot if selectroot is not None else sr, eshift=inp.eshift,
                  ras1=tuple(inp.ras1), ras2=tuple(inp.ras2), ras3=tuple(inp.ras3),
                  ras1_max_hole=inp.ras1_max_hole, ras3_max_elec=inp.ras3_max_elec,
                  min_hole_ras1=inp.min_hole_ras1, min_elec_ras3=inp.min_elec_ras3)


# ======================================================================================
# Two-electron integrals: 16-partner expansion of MDCINTNEW records into dense regions
# ======================================================================================
def expand_partners(idx1: np.ndarray, val: np.ndarray):
    """All (ij|kl) partners a record stands for (module_2integrals.F90:395-434).

    Returns (P, V): P (16, n, 4) 0-based indices, V (16, n) complex values.  Records with
    i == j and k > l are dropped as the reference's readers do (module_2integrals.F90:393,
    divide_2_elec_integral_into_subspaces.F90:117)."""
    i, j, k, l = (idx1[:, c].astype(np.int64) for c in range(4))
    keep = ~((i == j) & (k > l))
    i, j, k, l, v = i[keep], j[keep], k[keep], l[keep], val[keep]

    def tr(x):  # Kramers partner, 1-based: odd -> +1, even -> -1
        return np.where((x + 1) % 2 == 0, x + 1, x - 1)

    itr, jtr, ktr, ltr = tr(i), tr(j), tr(k), tr(l)
    sij = np.where((i + j) % 2 == 0, 1.0, -1.0)
    skl = np.where((k + l) % 2 == 0, 1.0, -1.0)
    vc = np.conj(v)
    P = [
        (i, j, k, l, v), (jtr, itr, k, l, v * sij), (i, j, ltr, ktr, v * skl), (jtr, itr, ltr, ktr, v * sij * skl),
        (j, i, l, k, vc), (itr, jtr, l, k, vc * sij), (j, i, ktr, ltr, vc * skl), (itr, jtr, ktr, ltr, vc * sij * skl),
        (k, l, i, j, v), (ltr, ktr, i, j, v * skl), (k, l, jtr, itr, v * sij), (ltr, ktr, jtr, itr, v * sij * skl),
        (l, k, j, i, vc), (ktr, ltr, j, i, vc * skl), (l, k, itr, jtr, vc * sij), (ktr, ltr, itr, jtr, vc * sij * skl),
    ]
    Pidx = np.stack([np.stack([a - 1, b - 1, c - 1, d - 1], axis=1) for (a, b, c, d, _) in P])
    Pval = np.stack([p[4] for p in P])
    return Pidx, Pval


class Integrals:
    """Dense two-electron integral blocks (pq|rs) in the ORIGINAL spinor basis, addressed
    by a space pattern (s1,s2,s3,s4) with s in {1,2,3}; '=' scatter semantics of the
    reference arrays (later partners overwrite earlier ones).  Records are expanded in
    chunks straight into the blocks the path reads."""

    PATTERNS = [(2, 1, 2, 2), (2, 1, 1, 1), (2, 1, 2, 1), (3, 2, 2, 2), (3, 2, 1, 1), (3, 1, 1, 2),
                (3, 1, 2, 2), (3, 2, 2, 1), (3, 1, 1, 1), (3, 1, 2, 1), (3, 2, 3, 2), (3, 1, 3, 2),
                (3, 1, 3, 1), (3, 3, 1, 1), (3, 3, 2, 2), (3, 1, 1, 3), (3, 2, 2, 3)]

    def __init__(self, sysm: System, chunk: int = 1 << 20):
        self.sysm = sysm
        nmoc = sysm.nmoc
        self._occ = np.zeros((nmoc,) * 4, dtype=np.complex128)
        self._cache: Dict[Tuple[int, ...], np.ndarray] = {}
        codes = {}
        for pat in self.PATTERNS:
            r = [self.rng(x) for x in pat]
            self._cache[pat] = np.zeros(tuple(b - a for a, b in r), dtype=np.complex128)
            codes[pat[0] * 1000 + pat[1] * 100 + pat[2] * 10 + pat[3]] = pat
        n = len(sysm.rec_val)
        for c0 in range(0, max(n, 1), chunk):
            P, V = expand_partners(sysm.rec_idx[c0:c0 + chunk], sysm.rec_val[c0:c0 + chunk])
            P = P.reshape(-1, 4)
            V = V.reshape(-1)
            sp = sysm.space_of(P).astype(np.int16)
            code = sp[:, 0] * 1000 + sp[:, 1] * 100 + sp[:, 2] * 10 + sp[:, 3]
            m = (sp <= 2).all(axis=1)              # every index inactive or active
            if np.any(m):
                q = P[m]
                self._occ[q[:, 0], q[:, 1], q[:, 2], q[:, 3]] = V[m]
            for cd, pat in codes.items():
                mm = code == cd
                if not np.any(mm):
                    continue
                q = P[mm]
                r = [self.rng(x) for x in pat]
                self._cache[pat][q[:, 0] - r[0][0], q[:, 1] - r[1][0], q[:, 2] - r[2][0], q[:, 3] - r[3][0]] = V[mm]

    def rng(self, s: int) -> Tuple[int, int]:
        ni, na, ns = self.sysm.ninact, self.sysm.nact, self.sysm.nsec
        return [(0, ni), (ni, ni + na), (ni + na, ni + na + ns)][s - 1]

    def block(self, pattern: Tuple[int, int, int, int]) -> np.ndarray:
        if pattern in self._cache:
            return self._cache[pattern]
        r = [self.rng(x) for x in pattern]
        if all(x <= 2 for x in pattern):
            return self._occ[r[0][0]:r[0][1], r[1][0]:r[1][1], r[2][0]:r[2][1], r[3][0]:r[3][1]]
        raise KeyError(f"integral block {pattern} is not read by the hot path")

    def occ_block(self) -> np.ndarray:
        """inttw(nmoc^4): every (pq|rs) with all indices inactive or active."""
        return self._occ


# ======================================================================================
# Determinant space and one-electron excitations
# ======================================================================================
def popcount(x: int) -> int:
    return bin(x).count("1")


def one_e_exct(I: int, c: int, a: int, nact: int):
    """E_{ca}|I> = phase * |J> (one_e_exct.F90:3-51); c, a 0-based.  None if zero."""
    if c == a:
        return (I, 0) if (I >> a) & 1 else None
    if not ((I >> a) & 1) or ((I >> c) & 1):
        return None
    J = I - (1 << a) + (1 << c)
    ia = ((1 << nact) - (1 << (a + 1))) if a + 1 < nact else 0
    ib = ((1 << nact) - (1 << (c + 1))) if c + 1 < nact else 0
    ph = popcount(I & ia) + popcount((I - (1 << a)) & ib)
    return J, ph


def ras_ok(I: int, s: System) -> bool:
    """ras_det_check.F90:1-59 applied by search_cas_configuration.F90:91-110."""
    if s.ras1:
        n1 = len(s.ras1)
        ne1 = popcount(I & ((1 << n1) - 1))
        if not (n1 - s.ras1_max_hole <= ne1 <= n1 - s.min_hole_ras1):
            return False
    if s.ras3:
        sh = len(s.ras1) + len(s.ras2)
        ne3 = popcount((I >> sh) << sh & I)
        if not (ne3 <= s.ras3_max_elec and s.min_elec_ras3 <= ne3):
            return False
    return True


def det_totsym(I: int, s: System) -> int:
    """cas_configuration_totsym (search_cas_configuration.F90:112-149)."""
    if s.nsymrpa == 1:
        return 1
    mds, md = s.multb_ds, s.multb_d
    ret = 1
    ielec = 0
    for t in range(s.nact):
        if (I >> t) & 1:
            ielec += 1
            jsym = int(s.irpamo[s.ninact + t])
            if ielec % 2 == 1:
                ret = int(mds[jsym - 1, ret - 1])
            else:
                partner = jsym + 1 if jsym % 2 == 1 else jsym - 1
                ret = int(md[partner - 1, ret - 1])
    if ielec % 2 == 0:
        ret += s.nsymrpa
    return ret


def enumerate_dets(s: System) -> List[int]:
    """search_cas_configuration.F90:3-110: Gosper order over nelec-of-nact bit strings."""
    out = []
    cur = (1 << s.nelec) - 1
    while cur < (1 << s.nact):
        if ras_ok(cur, s) and (s.nsymrpa == 1 or det_totsym(cur, s) == s.totsym):
            out.append(cur)
        t = (cur | (cur - 1)) + 1
        cur = t | ((((t & -t) // (cur & -cur)) >> 1) - 1)
    return out


# ======================================================================================
# CASCI (casmat.F90, diag.F90, casci.F90)
# ======================================================================================
def casmat(s: System, dets: List[int], g: np.ndarray) -> np.ndarray:
    """CASCI Hamiltonian by Slater-Condon rules (casmat.F90:3-222); g = inttw (nmoc^4)."""
    ni, na = s.ninact, s.nact
    ndet = len(dets)
    index = {d: n for n, d in enumerate(dets)}
    H = np.zeros((ndet, ndet), dtype=np.complex128)
    h = s.h
    for n, I in enumerate(dets):
        occ = [t for t in range(na) if (I >> t) & 1]
        vir = [t for t in range(na) if not (I >> t) & 1]
        occg = list(range(ni)) + [ni + t for t in occ]
        # diagonal (casmat.F90:54-104)
        d = sum(h[r, r] for r in occg)
        m0 = 0.0
        for x in range(len(occg)):
            r = occg[x]
            for y in range(x + 1, len(occg)):
                q = occg[y]
                m0 += 0.5 * g[r, r, q, q] - 0.5 * g[r, q, q, r]
        H[n, n] = d + m0 + np.conj(m0)
        # singles (casmat.F90:106-169)
        for r_ in occ:
            ir = ni + r_
            for a_ in vir:
                ia = ni + a_
                res = one_e_exct(I, a_, r_, na)
                if res is None or res[0] not in index:
                    continue
                m = index[res[0]]
                if m <= n:
                    continue
                val = h[ir, ia]
                for q in occg:
                    val += g[ir, ia, q, q] - g[ir, q, q, ia]
                val *= 1 if res[1] % 2 == 0 else -1
                H[n, m] = val
                H[m, n] = np.conj(val)
        # doubles (casmat.F90:170-213)
        for x in range(len(occ)):
            for y in range(x + 1, len(occ)):
                r_, q_ = occ[x], occ[y]
                for u in range(len(vir)):
                    for w in range(u + 1, len(vir)):
                        a_, b_ = vir[u], vir[w]
                        r1 = one_e_exct(I, a_, r_, na)
                        if r1 is None:
                            continue
                        r2 = one_e_exct(r1[0], b_, q_, na)
                        if r2 is None or r2[0] not in index:
                            continue
                        m = index[r2[0]]
                        if m <= n:
                            continue
                        ir, iq, ia, ib = ni + r_, ni + q_, ni + a_, ni + b_
                        val = g[ir, ia, iq, ib] - g[ir, ib, iq, ia]
                        val *= 1 if (r1[1] + r2[1]) % 2 == 0 else -1
                        H[n, m] = val
                        H[m, n] = np.conj(val)
    return H


def heev_upper(A: np.ndarray):
    """ZHEEV/DSYEV(jobz='V', uplo='U') semantics: only the upper triangle is referenced,
    eigenvalues ascending (diag.F90:43,109)."""
    return np.linalg.eigh(A, UPLO="U")


# ======================================================================================
# Densities
# ======================================================================================
class FullSpace:
    """The full N-electron active space (every nelec-of-nact bit string, Gosper order) with
    the CI vector embedded in it.  Intermediate determinants of the reference's
    ``dimN_density`` loops are unrestricted bit strings, so operator products are exact
    in this space (density_matrix.F90:3-247)."""

    def __init__(self, s: System, dets: List[int]):
        na, ne = s.nact, s.nelec
        full = []
        cur = (1 << ne) - 1
        while cur < (1 << na):
            full.append(cur)
            t = (cur | (cur - 1)) + 1
            cur = t | ((((t & -t) // (cur & -cur)) >> 1) - 1)
        self.full = full
        self.index = {d: n for n, d in enumerate(full)}
        self.ci_pos = np.array([self.index[d] for d in dets], dtype=np.int64)
        self.na = na
        M = len(full)
        # E_pq as sparse triplets: for each (p,q) arrays (src, dst, sign)
        self.ops = {}
        for p in range(na):
            for q in range(na):
                src, dst, sg = [], [], []
                for n, I in enumerate(full):
                    r = one_e_exct(I, p, q, na)
                    if r is None:
                        continue
                    src.append(n)
                    dst.append(self.index[r[0]])
                    sg.append(1.0 if r[1] % 2 == 0 else -1.0)
                self.ops[(p, q)] = (np.array(src, dtype=np.int64), np.array(dst, dtype=np.int64),
                                    np.array(sg))
        self.M = M

    def embed(self, c: np.ndarray) -> np.ndarray:
        psi = np.zeros((self.M,) + c.shape[1:], dtype=np.complex128)
        psi[self.ci_pos] = c
        return psi

    def apply(self, p: int, q: int, x: np.ndarray) -> np.ndarray:
        """y = E_pq x (x may carry trailing columns)."""
        src, dst, sg = self.ops[(p, q)]
        y = np.zeros_like(x)
        if len(src):   # E_pq maps determinants one to one: a plain scatter
            y[dst] = x[src] * sg.reshape((-1,) + (1,) * (x.ndim - 1))
        return y

    def project(self, x: np.ndarray) -> np.ndarray:
        """Zero components outside the CI space (final-determinant lookup of the reference)."""
        y = np.zeros_like(x)
        y[self.ci_pos] = x[self.ci_pos]
        return y


class RDM:
    """Dense <0|E..E|0> tensors for one CI vector (rdm mode).

    D1[a,b]      = <E_ab>                       (dim1_density)
    D2[a,b,c,d]  = <E_ab E_cd>                  (dim2_density)
    D3[...]      = <E_ab E_cd E_ef>             (dim3_density)
    T1/T2/T3     = same with sum_w eps_w E_ww rightmost (dim2/3/4_density(...,w,w) weighted)
    """

    def __init__(self, fs: FullSpace, c: np.ndarray, eps_act: Optional[np.ndarray] = None, order: int = 3):
        na = fs.na
        psi = fs.embed(c)
        bra = fs.project(psi)              # <0| lives in the CI space
        self.na = na
        Y = np.stack([fs.apply(p, q, psi) for p in range(na) for q in range(na)], axis=1)  # (M, na^2)
        # <0|E_ab X> = (E_ba ... ) : bra is the CI vector itself
        self.D1 = (np.conj(bra) @ Y).reshape(na, na)
        # D2[ab,cd] = sum_K conj( (E_ba psi)_K restricted ) ... use <0|E_ab = (E_ba |0>)^dagger
        Yb = np.stack([fs.apply(q, p, bra) for p in range(na) for q in range(na)], axis=1)  # col ab = E_ba bra
        self.D2 = (np.conj(Yb).T @ Y).reshape(na, na, na, na)
        if order >= 3:
            Z = np.stack([fs.apply(p, q, Y) for p in range(na) for q in range(na)], axis=1)  # (M, na^2, na^2)
            self.D3 = np.einsum("ka,kbc->abc", np.conj(Yb), Z).reshape((na,) * 6)
        if eps_act is not None:
            occ_e = np.array([sum(eps_act[t] for t in range(na) if (I >> t) & 1) for I in fs.full])
            psit = psi * occ_e
            Yt = np.stack([fs.apply(p, q, psit) for p in range(na) for q in range(na)], axis=1)
            self.T1 = (np.conj(bra) @ Yt).reshape(na, na)
            self.T2 = (np.conj(Yb).T @ Yt).reshape(na, na, na, na)
            if order >= 3:
                Zt = np.stack([fs.apply(p, q, Yt) for p in range(na) for q in range(na)], axis=1)
                self.T3 = np.einsum("ka,kbc->abc", np.conj(Yb), Zt).reshape((na,) * 6)
            self.e0_weights = occ_e


def density_literal(ops: List[Tuple[int, int]], dets: List[int], c: np.ndarray, na: int) -> complex:
    """<0|E_{c1a1} ... E_{cnan}|0> by the reference's determinant loop
    (density_matrix.F90:3-247); ops given left to right, applied right to left."""
    index = {d: n for n, d in enumerate(dets)}
    acc = 0.0 + 0.0j
    for n, I in enumerate(dets):
        cur, ph = I, 0
        ok = True
        for (cc, aa) in reversed(ops):
            r = one_e_exct(cur, cc, aa, na)
            if r is None:
                ok = False
                break
            cur, ph = r[0], ph + r[1]
        if not ok or cur not in index:
            continue
        m = index[cur]
        v = c[n] * np.conj(c[m])
        acc += v if ph % 2 == 0 else -v
    return acc


# ======================================================================================
# Fock matrix, its diagonalisation and the CI rotation
# ======================================================================================
def fock_casci(s: System, ints: Integrals, g_occ: np.ndarray, D1: np.ndarray) -> np.ndarray:
    """CASCI-state Fock matrix on the occ x occ and sec x sec blocks (fockcasci.F90:4-90)."""
    ni, na, ns, nmo = s.ninact, s.nact, s.nsec, s.nmo
    nmoc = ni + na
    f = np.zeros((nmo, nmo), dtype=np.complex128)
    Dt = np.zeros((nmoc, nmoc), dtype=np.complex128)
    Dt[np.arange(ni), np.arange(ni)] = 1.0
    Dt[ni:, ni:] = D1
    # occ block: h + sum_kl Dt_kl [(ij|kl) - (il|kj)]
    fo = s.h[:nmoc, :nmoc] + np.einsum("ijkl,kl->ij", g_occ, Dt) - np.einsum("ilkj,kl->ij", g_occ, Dt)
    iu = np.triu_indices(nmoc)
    fu = np.zeros_like(fo)
    fu[iu] = fo[iu]
    f[:nmoc, :nmoc] = fu + np.conj(np.triu(fu, 1)).T
    if ns:
        sl = slice(nmoc, nmoc + ns)
        fs_ = s.h[sl, sl].copy()
        # (ab|kl) with k,l occupied: patterns (3,3,1,1),(3,3,2,2) and (3,3,1,2),(3,3,2,1) are
        # absent from the reference (only diagonal-space pairs are stored); Dt is block diagonal.
        f1_11 = ints.block((3, 3, 1, 1))
        f1_22 = ints.block((3, 3, 2, 2))
        f2_11 = ints.block((3, 1, 1, 3))
        f2_22 = ints.block((3, 2, 2, 3))
        fs_ += np.einsum("abkk->ab", f1_11) - np.einsum("akkb->ab", f2_11)
        fs_ += np.einsum("abkl,kl->ab", f1_22, D1) - np.einsum("alkb,kl->ab", f2_22, D1)
        iu2 = np.triu_indices(ns)
        fu2 = np.zeros_like(fs_)
        fu2[iu2] = fs_[iu2]
        f[sl, sl] = fu2 + np.conj(np.triu(fu2, 1)).T
    return f


PAIR_DEGENERACY = 1e-10
TIE = 1e-8


def _first_near_max(x: np.ndarray) -> int:
    """Smallest index whose value is within a relative 1e-8 of the maximum."""
    m = float(np.max(x))
    return int(np.flatnonzero(x >= m - TIE * abs(m))[0])


def canonical_pairs(w: np.ndarray, V: np.ndarray) -> np.ndarray:
    """Canonical vectors inside exactly degenerate eigenvalue pairs.

    ZHEEV's choice of vectors inside a degenerate pair is decided by rounding, and the
    reference's complex E-space formula is not invariant under it.  For each pair (q,q+1)
    with |w_q+1 - w_q| <= 1e-10 max(1,|w_q|): v1 = P e_k / |P e_k| with k the first basis
    index of near-maximal P_kk (P the pair projector), v2 the unit vector of the pair
    orthogonal to v1 with its first near-largest component real positive."""
    V = V.copy()
    n = len(w)
    q = 0
    while q < n - 1:
        if abs(w[q + 1] - w[q]) <= PAIR_DEGENERACY * max(1.0, abs(w[q])):
            W = V[:, q:q + 2]
            pk = np.sum(np.abs(W) ** 2, axis=1)          # P_kk
            k = _first_near_max(pk)
            a = np.conj(W[k, :])
            a = a / np.linalg.norm(a)
            b = np.array([-np.conj(a[1]), np.conj(a[0])])
            v1 = W @ a
            v2 = W @ b
            l = _first_near_max(np.abs(v2))
            v2 = v2 * (np.conj(v2[l]) / abs(v2[l]))
            V[:, q], V[:, q + 1] = v1, v2
            q += 2
        else:
            q += 1
    return V


def fock_diag(s: System, f: np.ndarray):
    """fockdiag.F90:4-78 with cdiag0 (diag.F90:230-375): per space and irrep Hermitian
    eigendecomposition.  Returns (U, eps) with U block diagonal (column j = new spinor j)."""
    nmo = s.nmo
    U = np.zeros((nmo, nmo), dtype=np.complex128)
    eps = np.zeros(nmo)
    ranges = [(0, s.ninact), (s.ninact, s.nmoc), (s.nmoc, s.nmoc + s.nsec)]
    for (n0, n1) in ranges:
        if n1 <= n0:
            continue
        for sym in range(1, s.nsymrpa + 1):
            ind = [i for i in range(n0, n1) if s.irpamo[i] == sym]
            if not ind:
                continue
            blk = f[np.ix_(ind, ind)]
            # facsym(i,j) = fock(ind(i),ind(j)) for i >= j, then hermitian fill: lower triangle drives
            low = np.tril(blk)
            herm = low + np.conj(np.tril(low, -1)).T
            w, v = heev_upper(herm)
            if n0 == s.ninact and n1 == s.nmoc:      # active space: canonical degenerate pairs
                v = canonical_pairs(w, v)
            eps[ind] = w
            U[np.ix_(ind, ind)] = v
    return U, eps


def ci_rotate(s: System, dets: List[int], U_act: np.ndarray, c: np.ndarray) -> np.ndarray:
    """tracic (trac.F90:76-156) with detsc (sdet.F90:58-110): ds(k,k~) = det(U[occ_k, occ_k~]),
    then solve ds c' = c (ZGESV)."""
    nd = len(dets)
    if s.nelec == 0:
        return np.linalg.solve(np.ones((nd, nd), dtype=np.complex128), c)
    occ = np.array([[t for t in range(s.nact) if (I >> t) & 1] for I in dets], dtype=np.int64)   # (nd, ne)
    ds = np.zeros((nd, nd), dtype=np.complex128)
    for a in range(nd):
        # U[occ_a, occ_b] for every b at once: (nd, ne, ne)
        sub = U_act[occ[a][None, :, None], occ[:, None, :]]
        ds[a] = np.linalg.det(sub)
    return np.linalg.solve(ds, c)


# ======================================================================================
# Transformation (module_intra.F90, tramo.F90)
# ======================================================================================
def transform_block(blk: np.ndarray, U: np.ndarray, r: List[Tuple[int, int]]) -> np.ndarray:
    """(i'j'|k'l') = sum conj(U_ii') U_jj' conj(U_kk') U_ll' (ij|kl)  (module_intra.F90:130-277);
    the |x| <= 1e-15 write cutoff of each pass is applied after the full transformation."""
    Ui = U[r[0][0]:r[0][1], r[0][0]:r[0][1]]
    Uj = U[r[1][0]:r[1][1], r[1][0]:r[1][1]]
    Uk = U[r[2][0]:r[2][1], r[2][0]:r[2][1]]
    Ul = U[r[3][0]:r[3][1], r[3][0]:r[3][1]]
    x = np.einsum("ijkl,lL->ijkL", blk, Ul, optimize=True)
    x = np.einsum("ijkL,kK->ijKL", x, np.conj(Uk), optimize=True)
    x = np.einsum("ijKL,jJ->iJKL", x, Uj, optimize=True)
    x = np.einsum("iJKL,iI->IJKL", x, np.conj(Ui), optimize=True)
    x[np.abs(x) <= INTRA_CUTOFF] = 0.0
    return x


# ======================================================================================
# Subspace solver core (shared by A-G)
# ======================================================================================
def solve_block(S: np.ndarray, B: np.ndarray, Vcols: np.ndarray, alphas: np.ndarray):
    """S eigendecomposition with the 1e-8 cutoff (cdiag + ccutoff, cutoff.F90:37-70),
    X = U lambda^-1/2 (ulambda_s_half.F90:14-75), B' = X^H B X, its eigendecomposition,
    then e2 = -sum |W^H X^H v|^2/(alpha+w), sumc2 = sum |.|^2/(alpha+w)^2
    (solve_A_subspace.F90:149-261).  Vcols: (dimn, nouter)."""
    ws, us = heev_upper(S)
    keep = ws >= SMAT_LIN_DEP_THRESHOLD
    dimm = int(np.count_nonzero(keep))
    if dimm == 0:
        return 0.0, 0.0, 0
    X = us[:, keep] * (ws[keep] ** -0.5)
    Bp = np.conj(X).T @ B @ X
    wb, W = heev_upper(Bp)
    vc1 = np.conj(W).T @ (np.conj(X).T @ Vcols)          # (dimm, nouter)
    den = alphas[None, :] + wb[:, None]
    a2 = np.abs(vc1) ** 2
    e2 = -float(np.sum(a2 / den))
    sc2 = float(np.sum(a2 / den ** 2))
    return e2, sc2, dimm


def _kept(S: np.ndarray) -> int:
    """dimm of cdiag(S, ..., smat_lin_dep_threshold): eigenvalues at or above the cutoff."""
    return int(np.count_nonzero(heev_upper(S)[0] >= SMAT_LIN_DEP_THRESHOLD))


def herm_from_upper(A: np.ndarray) -> np.ndarray:
    u = np.triu(A)
    return u + np.conj(np.triu(u, 1)).T


# ======================================================================================
# Driver
# ======================================================================================
@dataclasses.dataclass
class Result:
    casci_energies: np.ndarray
    e0: float
    e2: Dict[str, float]
    sumc2: Dict[str, float]
    e2_sym: Dict[str, Dict[int, float]]
    total_energy: float
    ndet: int
    eps: np.ndarray

    @property
    def e2_total(self) -> float:
        return float(sum(self.e2.values()))

    @property
    def sumc2_total(self) -> float:
        return float(sum(self.sumc2.values()))


def run(s: System, mode: str = "rdm", subspaces: str = SUBSPACES, verbose: bool = False,
        active_pair_rotation: Optional[np.random.Generator] = None, lean: bool = False) -> Result:
    """r4dcasci (r4dcasci.F90:1-134) followed by r4dcaspt2_tra (r4dcaspt2_tra.F90:4-482).

    ``active_pair_rotation``: when given, the eigenvectors of every exactly degenerate pair of
    active Fock eigenvalues are rotated by a random unitary 2x2 matrix.  Such a rotation is
    an equally valid ZHEEV result; every subspace except E is invariant under it (see
    ``e_subspace_envelope``).

    ``lean``: release memory as soon as it is no longer read (for the largest systems): the
    record arrays of ``s`` after the integral expansion (``s.rec_idx``/``s.rec_val`` become
    empty), the Fock-only blocks after the Fock build, and each original-basis class block once
    it has been transformed.  The numbers are the same."""
    ni, na, ns = s.ninact, s.nact, s.nsec
    nmoc = ni + na
    ints = Integrals(s)
    if lean:
        s.rec_idx = np.zeros((0, 4), np.int32)
        s.rec_val = np.zeros(0, np.complex128)
    g_occ = ints.occ_block()
    dets = enumerate_dets(s)
    ndet = len(dets)
    if ndet == 0:
        raise ValueError("no CASCI configuration for this totsym")
    H = casmat(s, dets, g_occ)
    w, v = heev_upper(H)
    eigen = w + s.ecore                                           # casci.F90:72
    iroot = s.selectroot - 1
    c0 = v[:, iroot].copy()
    fs = FullSpace(s, dets)

    # ---- Fock matrix of the CASCI state and its diagonalisation
    rd_c = RDM(fs, c0, order=1)
    f = fock_casci(s, ints, g_occ, rd_c.D1)
    if lean:   # blocks only the Fock build reads
        for pat in ((3, 3, 1, 1), (3, 3, 2, 2), (3, 1, 1, 3), (3, 2, 2, 3)):
            ints._cache.pop(pat, None)
    U, eps = fock_diag(s, f)
    if active_pair_rotation is not None:
        for p in range(ni, nmoc - 1):
            if abs(eps[p] - eps[p + 1]) <= 1e-12 * max(1.0, abs(eps[p])):
                g = active_pair_rotation
                M2 = g.normal(size=(2, 2)) + (0.0 if s.realonly else 1j * g.normal(size=(2, 2)))
                Q, _ = np.linalg.qr(M2)   # real systems: DSYEV vectors are real (orthogonal Q)
                U[:, p:p + 2] = U[:, p:p + 2] @ Q
    c = ci_rotate(s, dets, U[ni:nmoc, ni:nmoc], c0)
    eps_act = eps[ni:nmoc]
    rd = RDM(fs, c, eps_act=eps_act, order=3)
    e0 = float(np.real(np.sum(np.diag(rd.D1) * eps_act)))          # calce0.F90:4-50

    # ---- transformed integral classes (local indices)
    cls = {}
    patterns = {"A1": (2, 1, 2, 2), "A2": (2, 1, 1, 1), "B": (2, 1, 2, 1), "C1": (3, 2, 2, 2),
                "C2": (3, 2, 1, 1), "C3": (3, 1, 1, 2), "D1": (3, 1, 2, 2), "D2": (3, 2, 2, 1),
                "D3": (3, 1, 1, 1), "E": (3, 1, 2, 1), "F": (3, 2, 3, 2), "G": (3, 1, 3, 2),
                "H": (3, 1, 3, 1)}
    for name, pat in patterns.items():
        cls[name] = transform_block(ints.block(pat), U, [ints.rng(p) for p in pat])
        if lean:
            ints._cache.pop(pat, None)
    hU = np.conj(U).T @ s.h @ U                                       # tramo1 (tramo.F90:4-68)

    res_e2, res_sc2, res_sym = {}, {}, {}
    kw = dict(s=s, rd=rd, cls=cls, hU=hU, eps=eps, e0=e0)
    for X in SUBSPACES:
        skip = (X in "ABDEGH" and ni == 0) or (X in "CDEFGH" and ns == 0)
        if skip or X not in subspaces:
            continue
        e2, sc2, per = SOLVERS[X](**kw)
        res_e2[X], res_sc2[X], res_sym[X] = e2, sc2, per
        if verbose:
            print(f" e2{X.lower()} = {e2: .15e}  sumc2,{X.lower()} = {sc2: .15e}")
    e2all = sum(res_e2.values())
    sumc2 = sum(res_sc2.values())
    total = e2all + float(eigen[iroot]) - s.eshift * sumc2               # r4dcaspt2_tra.F90:437-442
    return Result(casci_energies=eigen, e0=e0, e2=res_e2, sumc2=res_sc2, e2_sym=res_sym,
                  total_energy=total, ndet=ndet, eps=eps)


# --------------------------------------------------------------------------------------
# helpers for the solvers
# --------------------------------------------------------------------------------------
def _md(s, a, b):
    return int(s.multb_d[a - 1, b - 1])


def _ms(s, a, b):
    return int(s.multb_s[a - 1, b - 1])


def _kp(x):
    """irrep of the Kramers partner: irpamo - (-1)**mod(irpamo,2)."""
    return x + 1 if x % 2 == 1 else x - 1


# --------------------------------------------------------------------------------------
# A: E_ti E_uv|0>  (solve_A_subspace.F90:26-678)
# --------------------------------------------------------------------------------------
def solve_A(s, rd, cls, hU, eps, e0):
    ni, na = s.ninact, s.nact
    gi = lambda t: ni + t
    A1, A2 = cls["A1"], cls["A2"]
    # effh(p,i) = tramo1(p,i) + sum_{k != i}[(pi|kk) - (pk|ki)]   (vAmat 546-631)
    effh = hU[ni:ni + na, :ni].copy()
    for i in range(ni):
        for k in range(ni):
            if k == i:
                continue
            effh[:, i] += A2[:, i, k, k] - A2[:, k, k, i]
    D1, D2, D3 = rd.D1, rd.D2, rd.D3
    V = (-np.einsum("piqr,vuptqr->ituv", A1, D3, optimize=True)
         + np.einsum("tipq,vupq->ituv", A1, D2, optimize=True)
         + np.einsum("ti,vu->ituv", effh, D1, optimize=True)
         - np.einsum("pi,vupt->ituv", effh, D2, optimize=True))
    e2_tot, sc2_tot, per = 0.0, 0.0, {}
    for isym in range(1, s.nsymrpa + 1):
        ind = []
        for x in range(na):
            for y in range(na):
                for z in range(na):
                    if s.nsymrpa == 1 or _ms(s, _md(s, s.irpamo[gi(x)], isym), _md(s, s.irpamo[gi(y)], s.irpamo[gi(z)])) == 1:
                        ind.append((x, y, z))
        if not ind:
            continue
        ind = np.array(ind)
        x, y, z = ind[:, 0], ind[:, 1], ind[:, 2]
        t, u, v = x, y, z
        Sm = (-D3[z[:, None], y[:, None], t[None, :], x[:, None], u[None, :], v[None, :]]
              + (t[None, :] == x[:, None]) * D2[z[:, None], y[:, None], u[None, :], v[None, :]])
        e = eps[gi(u)] + eps[gi(t)] - eps[gi(v)]
        Bm = (-rd.T3[z[:, None], y[:, None], t[None, :], x[:, None], u[None, :], v[None, :]]
              + (t[None, :] == x[:, None]) * rd.T2[z[:, None], y[:, None], u[None, :], v[None, :]]
              + Sm * e[None, :])
        Sm, Bm = herm_from_upper(Sm), herm_from_upper(Bm)
        outer = [i for i in range(ni) if s.nsymrpa == 1 or s.irpamo[i] == isym]
        if not outer:
            # the reference still diagonalises S and prints a zero e2X(isym) when it keeps
            # vectors (solve_A_subspace.F90:155-164,262)
            if _kept(Sm):
                per[isym] = 0.0
            continue
        Vc = V[np.array(outer)][:, x, y, z].T
        alphas = np.array([-eps[i] - e0 + s.eshift for i in outer])
        e2, sc2, dimm = solve_block(Sm, Bm, Vc, alphas)
        if dimm:   # printed only for a kept dimension (solve_A_subspace.F90:158-164)
            per[isym] = e2
        e2_tot += e2
        sc2_tot += sc2
    return e2_tot, sc2_tot, per


# --------------------------------------------------------------------------------------
# B: E_ti E_uj|0>, t>u, i>j  (solve_B_subspace.F90:27-591)
# --------------------------------------------------------------------------------------
def solve_B(s, rd, cls, hU, eps, e0):
    ni, na = s.ninact, s.nact
    gi = lambda t: ni + t
    Bc = cls["B"]                       # (t i|u j)
    D1, D2 = rd.D1, rd.D2
    # V(ij;x,y) for i>j from records R[t,u] = (t i|u j)   (vBmat_complex)
    R = np.einsum("tiuj->ijtu", Bc)
    V = (R - np.einsum("ijyx->ijxy", R)
         + np.einsum("ijyu,ux->ijxy", R, D1) - np.einsum("ijxu,uy->ijxy", R, D1)
         - np.einsum("ijty,tx->ijxy", R, D1)
         + np.einsum("ijtu,txuy->ijxy", R, D2, optimize=True))
    pairs = [(i, j) for i in range(ni) for j in range(i)]
    e2_tot, sc2_tot, per = 0.0, 0.0, {}
    for isym in range(1, s.nsymrpa + 1):
        ind = [(t, u) for t in range(na) for u in range(t)
               if s.nsymrpa == 1 or _md(s, s.irpamo[gi(t)], _kp(s.irpamo[gi(u)])) == isym]
        if not ind:
            continue
        ind = np.array(ind)
        x, y = ind[:, 0], ind[:, 1]
        t, u = x[None, :], y[None, :]
        X_, Y_ = x[:, None], y[:, None]
        Sm = (D2[t, X_, u, Y_] - (t == X_) * D1[u, Y_] - (u == Y_) * D1[t, X_] - (t == Y_) * D1[u, X_]
              + ((t == X_) & (u == Y_)))
        e = eps[gi(x)] + eps[gi(y)]
        Bm = (rd.T2[t, X_, u, Y_] - (t == X_) * rd.T1[u, Y_] - (u == Y_) * rd.T1[t, X_] - (t == Y_) * rd.T1[u, X_]
              + ((t == X_) & (u == Y_)) * e0 + Sm * e[None, :])
        Sm, Bm = herm_from_upper(Sm), herm_from_upper(Bm)
        outer = [(i, j) for (i, j) in pairs
                 if s.nsymrpa == 1 or _ms(s, _md(s, _kp(s.irpamo[i]), s.irpamo[j]), isym) == 1]
        if not outer:
            # the reference still diagonalises S and prints a zero e2X(isym) when it keeps
            # vectors (solve_A_subspace.F90:155-164,262)
            if _kept(Sm):
                per[isym] = 0.0
            continue
        Vc = np.stack([V[i, j][x, y] for (i, j) in outer], axis=1)
        alphas = np.array([-eps[i] - eps[j] - e0 + s.eshift for (i, j) in outer])
        e2, sc2, dimm = solve_block(Sm, Bm, Vc, alphas)
        if dimm:   # printed only for a kept dimension (solve_A_subspace.F90:158-164)
            per[isym] = e2
        e2_tot += e2
        sc2_tot += sc2
    return e2_tot, sc2_tot, per


# --------------------------------------------------------------------------------------
# C: E_at E_uv|0>  (solve_C_subspace.F90:26-658)
# --------------------------------------------------------------------------------------
def solve_C(s, rd, cls, hU, eps, e0):
    ni, na, ns = s.ninact, s.nact, s.nsec
    nmoc = ni + na
    gi = lambda t: ni + t
    C1, C2, C3 = cls["C1"], cls["C2"], cls["C3"]
    effh = hU[nmoc:nmoc + ns, ni:nmoc].copy()                 # tramo1(a,t)
    effh -= np.einsum("aqqp->ap", C1)
    effh += np.einsum("apkk->ap", C2)
    effh -= np.einsum("akkp->ap", C3)
    effh[np.abs(effh) < EFFH_C_SKIP] = 0.0
    D2, D3 = rd.D2, rd.D3
    V = (np.einsum("ajkl,vutjkl->atuv", C1, D3, optimize=True)
         + np.einsum("ap,vutp->atuv", effh, D2, optimize=True))
    e2_tot, sc2_tot, per = 0.0, 0.0, {}
    for isym in range(1, s.nsymrpa + 1):
        ind = []
        for x in range(na):
            for y in range(na):
                for z in range(na):
                    if s.nsymrpa == 1 or _ms(s, _md(s, isym, s.irpamo[gi(x)]), _md(s, s.irpamo[gi(y)], s.irpamo[gi(z)])) == 1:
                        ind.append((x, y, z))
        if not ind:
            continue
        ind = np.array(ind)
        x, y, z = ind[:, 0], ind[:, 1], ind[:, 2]
        t, u, v = x[None, :], y[None, :], z[None, :]
        Sm = D3[z[:, None], y[:, None], x[:, None], t, u, v]
        e = eps[gi(y)] - eps[gi(z)] - eps[gi(x)]
        Bm = rd.T3[z[:, None], y[:, None], x[:, None], t, u, v] + Sm * e[None, :]
        Sm, Bm = herm_from_upper(Sm), herm_from_upper(Bm)
        outer = [a for a in range(ns) if s.nsymrpa == 1 or s.irpamo[nmoc + a] == isym]
        if not outer:
            # the reference still diagonalises S and prints a zero e2X(isym) when it keeps
            # vectors (solve_A_subspace.F90:155-164,262)
            if _kept(Sm):
                per[isym] = 0.0
            continue
        Vc = V[np.array(outer)][:, x, y, z].T
        alphas = np.array([eps[nmoc + a] - e0 + s.eshift for a in outer])
        e2, sc2, dimm = solve_block(Sm, Bm, Vc, alphas)
        if dimm:   # printed only for a kept dimension (solve_A_subspace.F90:158-164)
            per[isym] = e2
        e2_tot += e2
        sc2_tot += sc2
    return e2_tot, sc2_tot, per


# --------------------------------------------------------------------------------------
# D: E_ai E_tu|0>  (solve_D_subspace.F90:25-609)
# --------------------------------------------------------------------------------------
def solve_D(s, rd, cls, hU, eps, e0):
    ni, na, ns = s.ninact, s.nact, s.nsec
    nmoc = ni + na
    gi = lambda t: ni + t
    D1c, D2c, D3c = cls["D1"], cls["D2"], cls["D3"]
    effh = hU[nmoc:nmoc + ns, :ni].copy()
    for i in range(ni):
        for k in range(ni):
            if k == i:
                continue
            effh[:, i] += D3c[:, i, k, k] - D3c[:, k, k, i]
    D1, D2 = rd.D1, rd.D2
    V = (np.einsum("aikl,utkl->aitu", D1c, D2, optimize=True)
         - np.einsum("ajki,utkj->aitu", D2c, D2, optimize=True)
         + np.einsum("ai,ut->aitu", effh, D1))
    e2_tot, sc2_tot, per = 0.0, 0.0, {}
    for isym in range(1, s.nsymrpa + 1):
        ind = [(t, u) for t in range(na) for u in range(na)
               if s.nsymrpa == 1 or _md(s, s.irpamo[gi(t)], s.irpamo[gi(u)]) == isym]
        if not ind:
            continue
        ind = np.array(ind)
        x, y = ind[:, 0], ind[:, 1]
        t, u = x[None, :], y[None, :]
        Sm = D2[y[:, None], x[:, None], t, u]
        e = eps[gi(x)] - eps[gi(y)]
        Bm = rd.T2[y[:, None], x[:, None], t, u] + Sm * e[None, :]
        Sm, Bm = herm_from_upper(Sm), herm_from_upper(Bm)
        outer = [(a, i) for a in range(ns) for i in range(ni)
                 if s.nsymrpa == 1 or _ms(s, _md(s, s.irpamo[nmoc + a], s.irpamo[i]), isym) == 1]
        if not outer:
            # the reference still diagonalises S and prints a zero e2X(isym) when it keeps
            # vectors (solve_A_subspace.F90:155-164,262)
            if _kept(Sm):
                per[isym] = 0.0
            continue
        Vc = np.stack([V[a, i][x, y] for (a, i) in outer], axis=1)
        alphas = np.array([eps[nmoc + a] - eps[i] - e0 + s.eshift for (a, i) in outer])
        e2, sc2, dimm = solve_block(Sm, Bm, Vc, alphas)
        if dimm:   # printed only for a kept dimension (solve_A_subspace.F90:158-164)
            per[isym] = e2
        e2_tot += e2
        sc2_tot += sc2
    return e2_tot, sc2_tot, per


# --------------------------------------------------------------------------------------
# E: E_ti E_aj|0>, i>j  (solve_E_subspace.F90:26-476)
# --------------------------------------------------------------------------------------
def solve_E(s, rd, cls, hU, eps, e0):
    ni, na, ns = s.ninact, s.nact, s.nsec
    nmoc = ni + na
    gi = lambda t: ni + t
    Ec = cls["E"]                              # (a i|p j)
    D1 = rd.D1
    # V(a,i>j;t) = -(ai|tj) + (aj|ti) + sum_p D1[t,p][(ai|pj) - (aj|pi)]
    W = Ec - np.einsum("ajpi->aipj", Ec)       # (ai|pj) - (aj|pi)
    V = -np.einsum("aitj->aijt", W) + np.einsum("tp,aipj->aijt", D1, W)
    e2_tot, sc2_tot, per = 0.0, 0.0, {}
    trip = [(i, j, a) for i in range(ni) for j in range(i) for a in range(ns)]
    for isym in range(1, s.nsymrpa + 1):
        ind = np.array([t for t in range(na) if s.irpamo[gi(t)] == isym], dtype=np.int64)
        if len(ind) == 0:
            continue
        Sm = np.eye(len(ind)) - D1[ind[None, :], ind[:, None]]
        Bm = -rd.T1[ind[None, :], ind[:, None]] + np.eye(len(ind)) * e0 + Sm * eps[gi(ind)][None, :]
        Sm, Bm = herm_from_upper(Sm), herm_from_upper(Bm)
        outer = [(i, j, a) for (i, j, a) in trip
                 if s.nsymrpa == 1 or _ms(s, _md(s, isym, s.irpamo[i]), _md(s, s.irpamo[nmoc + a], s.irpamo[j])) == 1]
        if not outer:
            # the reference still diagonalises S and prints a zero e2X(isym) when it keeps
            # vectors (solve_A_subspace.F90:155-164,262)
            if _kept(Sm):
                per[isym] = 0.0
            continue
        Vc = np.stack([V[a, i, j][ind] for (i, j, a) in outer], axis=1)
        alphas = np.array([eps[nmoc + a] - eps[i] - eps[j] - e0 + s.eshift for (i, j, a) in outer])
        e2, sc2, dimm = solve_block(Sm, Bm, Vc, alphas)
        if dimm:   # printed only for a kept dimension (solve_A_subspace.F90:158-164)
            per[isym] = e2
        e2_tot += e2
        sc2_tot += sc2
    return e2_tot, sc2_tot, per


# --------------------------------------------------------------------------------------
# F: E_at E_bu|0>, a>b, t>u  (solve_F_subspace.F90:26-544)
# --------------------------------------------------------------------------------------
def solve_F(s, rd, cls, hU, eps, e0):
    ni, na, ns = s.ninact, s.nact, s.nsec
    nmoc = ni + na
    gi = lambda t: ni + t
    Fc = cls["F"]                              # (a p|b q)
    D1, D2 = rd.D1, rd.D2
    V = (np.einsum("apbq,xpyq->abxy", Fc, D2, optimize=True)
         - np.einsum("aybq,xq->abxy", Fc, D1, optimize=True))
    e2_tot, sc2_tot, per = 0.0, 0.0, {}
    pairs = [(a, b) for a in range(ns) for b in range(a)]
    for isym in range(1, s.nsymrpa + 1):
        ind = [(t, u) for t in range(na) for u in range(t)
               if s.nsymrpa == 1 or _md(s, _kp(s.irpamo[gi(u)]), s.irpamo[gi(t)]) == isym]
        if not ind:
            continue
        ind = np.array(ind)
        vv, xx = ind[:, 0], ind[:, 1]             # row (v,x), column (t,u)
        t, u = vv[None, :], xx[None, :]
        V_, X_ = vv[:, None], xx[:, None]
        Sm = D2[V_, t, X_, u] - (X_ == t) * D1[V_, u]
        e = -eps[gi(xx)] - eps[gi(vv)]
        Bm = rd.T2[V_, t, X_, u] - (X_ == t) * rd.T1[V_, u] + Sm * e[None, :]
        Sm, Bm = herm_from_upper(Sm), herm_from_upper(Bm)
        outer = [(a, b) for (a, b) in pairs
                 if s.nsymrpa == 1 or _ms(s, _md(s, s.irpamo[nmoc + a], _kp(s.irpamo[nmoc + b])), isym) == 1]
        if not outer:
            # the reference still diagonalises S and prints a zero e2X(isym) when it keeps
            # vectors (solve_A_subspace.F90:155-164,262)
            if _kept(Sm):
                per[isym] = 0.0
            continue
        Vc = np.stack([V[a, b][vv, xx] for (a, b) in outer], axis=1)
        alphas = np.array([eps[nmoc + a] + eps[nmoc + b] - e0 + s.eshift for (a, b) in outer])
        e2, sc2, dimm = solve_block(Sm, Bm, Vc, alphas)
        if dimm:   # printed only for a kept dimension (solve_A_subspace.F90:158-164)
            per[isym] = e2
        e2_tot += e2
        sc2_tot += sc2
    return e2_tot, sc2_tot, per


# --------------------------------------------------------------------------------------
# G: E_ai E_bt|0>, a>b  (solve_G_subspace.F90:26-469)
# --------------------------------------------------------------------------------------
def solve_G(s, rd, cls, hU, eps, e0):
    ni, na, ns = s.ninact, s.nact, s.nsec
    nmoc = ni + na
    gi = lambda t: ni + t
    Gc = cls["G"]                              # (a i|b p)
    D1 = rd.D1
    W = Gc - np.einsum("biap->aibp", Gc)       # (ai|bp) - (bi|ap)
    V = np.einsum("tp,aibp->abit", D1, W)
    e2_tot, sc2_tot, per = 0.0, 0.0, {}
    trip = [(a, b, i) for a in range(ns) for b in range(a) for i in range(ni)]
    for isym in range(1, s.nsymrpa + 1):
        ind = np.array([t for t in range(na) if s.irpamo[gi(t)] == isym], dtype=np.int64)
        if len(ind) == 0:
            continue
        Sm = D1[ind[:, None], ind[None, :]]
        Bm = rd.T1[ind[:, None], ind[None, :]] - Sm * eps[gi(ind)][:, None]
        Sm, Bm = herm_from_upper(Sm), herm_from_upper(Bm)
        outer = [(a, b, i) for (a, b, i) in trip
                 if s.nsymrpa == 1 or _ms(s, _md(s, s.irpamo[nmoc + b], isym), _md(s, s.irpamo[nmoc + a], s.irpamo[i])) == 1]
        if not outer:
            # the reference still diagonalises S and prints a zero e2X(isym) when it keeps
            # vectors (solve_A_subspace.F90:155-164,262)
            if _kept(Sm):
                per[isym] = 0.0
            continue
        Vc = np.stack([V[a, b, i][ind] for (a, b, i) in outer], axis=1)
        alphas = np.array([-eps[i] + eps[nmoc + a] + eps[nmoc + b] - e0 + s.eshift for (a, b, i) in outer])
        e2, sc2, dimm = solve_block(Sm, Bm, Vc, alphas)
        if dimm:   # printed only for a kept dimension (solve_A_subspace.F90:158-164)
            per[isym] = e2
        e2_tot += e2
        sc2_tot += sc2
    return e2_tot, sc2_tot, per


# --------------------------------------------------------------------------------------
# H: E_ai E_bj|0>, a>b, i>j  (solve_H_subspace.F90:23-191)
# --------------------------------------------------------------------------------------
def solve_H(s, rd, cls, hU, eps, e0):
    ni, na, ns = s.ninact, s.nact, s.nsec
    nmoc = ni + na
    Hc = cls["H"]                              # (a i|b j)
    V = Hc - np.einsum("ajbi->aibj", Hc)       # (ai|bj) - (aj|bi)
    e2, sc2 = 0.0, 0.0
    ea = eps[nmoc:nmoc + ns]
    ei = eps[:ni]
    a_, b_ = np.tril_indices(ns, -1)
    i_, j_ = np.tril_indices(ni, -1)
    Vab = V[a_[:, None], i_[None, :], b_[:, None], j_[None, :]]
    den = ea[a_][:, None] + ea[b_][:, None] - ei[i_][None, :] - ei[j_][None, :] + s.eshift
    ir = np.asarray(s.irpamo)
    md, msy = s.multb_d, s.multb_s
    s1 = md[ir[nmoc + a_][:, None] - 1, ir[i_][None, :] - 1]
    s2 = md[ir[nmoc + b_][:, None] - 1, ir[j_][None, :] - 1]
    mask = msy[s1 - 1, s2 - 1] == 1
    c = Vab / den
    sc2 = float(np.sum((np.abs(c) ** 2)[mask]))
    e2 = -float(np.sum((np.abs(Vab) ** 2 / den)[mask]))
    return e2, sc2, {}


def e_subspace_envelope(s: System, trials: int = 6, seed: int = 0) -> Tuple[float, float]:
    """Range of the E-subspace energy over equally valid eigenvector choices inside
    degenerate active Kramers pairs.

    The reference's complex E-space V build (solve_E_subspace.F90 vEmat_complex) contracts
    the integrals with dim1_density(it, k) = <E_tp>; covariance under a phase change of the
    active spinors would need <E_pt>.  For real integrals the two are equal; for complex
    integrals without point-group symmetry the active Fock block has exactly degenerate
    Kramers pairs, ZHEEV's choice of vectors inside a pair is decided by rounding, and so
    the reference's e2E is defined only to within this range."""
    vals = [run(s, subspaces="E").e2.get("E", 0.0)]
    g = np.random.default_rng(seed)
    for _ in range(trials):
        vals.append(run(s, subspaces="E", active_pair_rotation=g).e2.get("E", 0.0))
    return float(min(vals)), float(max(vals))


SOLVERS = {"A": solve_A, "B": solve_B, "C": solve_C, "D": solve_D,
           "E": solve_E, "F": solve_F, "G": solve_G, "H": solve_H}


# ======================================================================================
# IVO: improved virtual orbitals (r4divo.F90, fockivo.F90)
# ======================================================================================
def ivo_fock(s: System, ints: Integrals, mo_energy: np.ndarray, nhomo: int) -> Tuple[np.ndarray, int]:
    """The Fock matrix of the secondary spinors for IVO (fockivo.F90:44-85):
    f(i,j) = e_i delta_ij - sum_k w_k [(ij|kk) - (ik|kj)] / numh over the numh highest active
    spinors k (w_k = 1/2 for the two highest when nelec is odd); numh = nhomo, or when 0 the
    number of spinors up to the last active one whose energy lies within 0.1 Eh of the HOMO
    e(ninact + nelec).  Only the upper triangle and the real diagonal are used downstream."""
    ni, na, ns = s.ninact, s.nact, s.nsec
    act_end = ni + na   # 1-based global index of the last active spinor
    if nhomo == 0:
        numh = int(np.count_nonzero(np.abs(mo_energy[:act_end] - mo_energy[s.nelec + ni - 1]) < 1.0e-1))
    else:
        numh = nhomo
    F1 = ints.block((3, 3, 2, 2))   # (ab|kl)
    F2 = ints.block((3, 2, 2, 3))   # (ak|lb)
    f = np.zeros((ns, ns), dtype=np.complex128)
    for i in range(ns):
        f[i, i] = mo_energy[act_end + i]
    for k in range(act_end - numh + 1, act_end + 1):   # 1-based global
        ka = k - 1 - ni
        w = 0.5 if (k > act_end - 2 and s.nelec % 2 == 1) else 1.0
        f += w * (-F1[:, :, ka, ka] + F2[:, ka, ka, :]) / numh
    return np.triu(f), numh


def ivo_blocks(s: System, nfsym: int) -> List[Tuple[int, np.ndarray]]:
    """(isym, secondary indices) of the blocks fockivo diagonalises (fockivo.F90:180-215):
    per fermion-irrep group, every second abelian irrep (one of each Kramers pair)."""
    out = []
    ni, na, ns = s.ninact, s.nact, s.nsec
    irp = np.asarray(s.irpamo[ni + na:ni + na + ns])
    for g in range(nfsym):
        start, end = (1, s.nsymrpa // 2) if g == 0 else (s.nsymrpa // 2 + 1, s.nsymrpa)
        for isym in range(start, end + 1, 2):
            out.append((isym, np.flatnonzero(irp == isym)))
    return out


def ivo(s: System, ints: Integrals, mo_energy: np.ndarray, d, nhomo: int, occ_mo_num, vcut_mo_num,
        lartg: str = "old"):
    """IVO (r4divo.F90:80-93, fockivo.F90:44-270): the virtual-space Fock matrix, its
    eigenvectors per abelian irrep block, and the DFPCMO coefficients of the virtual MOs
    rotated by them.  Returns (new coefficient vector, {isym: eigenvalues}, numh)."""
    fu, numh = ivo_fock(s, ints, mo_energy, nhomo)
    coef = d.coef.copy()
    mo = [p + e for p, e in zip(d.positronic, d.electronic)]
    evals = {}
    blocks = ivo_blocks(s, d.nfsym)
    for g in range(d.nfsym):
        nao = d.basis_ao[g]
        base = (0 if g == 0 else d.basis_all[0]) + (d.positronic[g] + occ_mo_num[g]) * nao
        nvirt = d.electronic[g] - occ_mo_num[g] - vcut_mo_num[g]
        itrfmo = coef[base:base + nvirt * nao].reshape(nvirt, nao).T.astype(np.complex128)   # (ao, mo)
        mo_off = (0 if g == 0 else mo[0]) + d.positronic[g] + occ_mo_num[g]
        lo = mo_off + 1
        hi = (0 if g == 0 else mo[0]) + d.positronic[g] + d.electronic[g] - vcut_mo_num[g]
        for isym, sec in blocks:
            if (g == 0) != (isym <= s.nsymrpa // 2):
                continue
            isym_sup = isym if g == 0 else isym - s.nsymrpa // 2
            sup = d.supersym[lo - 1:hi]
            if np.all(sup == 0):
                dmosym = np.arange(lo, hi + 1)
            else:
                dmosym = np.arange(lo, hi + 1)[np.abs(sup) == isym_sup]
            nv = len(sec)
            fs = fu[np.ix_(sec, sec)]
            A = np.triu(fs, 1)
            A = A + A.conj().T + np.diag(fs.diagonal().real)
            w, V = zheev_lapack(A, lartg)
            evals[isym] = w
            cols = dmosym - mo_off - 1
            if len(cols) != nv:
                raise ValueError("IVO: DFPCMO and input disagree on the virtual MOs of an irrep")
            itrfmo[:, cols] = itrfmo[:, cols] @ V
        coef[base:base + nvirt * nao] = itrfmo.real.T.reshape(-1)
    return coef, evals, numh


# ======================================================================================
# LAPACK ZHEEV, restated step by step (the eigenvector signs of IVO's DFPCMONEW)
# ======================================================================================
# The IVO orbitals are ZHEEV's eigenvectors (diag.F90:66-128 cdiag, jobz 'V', uplo 'U'), and
# the sign of each is whatever that algorithm leaves.  This restates the published LAPACK
# 3.x reference algorithm (not in the reference project; a link-time dependency): ZHETD2
# (Householder reduction, upper), ZUNGTR/ZUNG2L (accumulate Q), ZSTEQR (implicit QL/QR
# with Wilkinson shifts, DLAEV2 for 2x2 blocks, selection sort).  Two generations of the
# Givens generator DLARTG differ in the sign of the rotation when |f| <= |g|, f < 0 (LAPACK
# <= 3.9 versus >= 3.10); ``lartg`` selects one.
_EPS = np.finfo(np.float64).eps * 0.5        # dlamch('E')
_SAFMIN = np.finfo(np.float64).tiny          # dlamch('S')


def _dlapy2(x, y):
    w, z = max(abs(x), abs(y)), min(abs(x), abs(y))
    return w if z == 0.0 else w * math.sqrt(1.0 + (z / w) ** 2)


def _dlartg(f, g, variant):
    if variant == "new":   # LAPACK >= 3.10 (la_xlartg)
        if g == 0.0:
            return 1.0, 0.0, f
        if f == 0.0:
            return 0.0, math.copysign(1.0, g), abs(g)
        d = math.sqrt(f * f + g * g)
        r = math.copysign(d, f)
        return abs(f) / d, g / r, r
    if g == 0.0:           # LAPACK <= 3.9
        return 1.0, 0.0, f
    if f == 0.0:
        return 0.0, 1.0, g
    r = math.sqrt(f * f + g * g)
    cs, sn = f / r, g / r
    if abs(f) > abs(g) and cs < 0.0:
        cs, sn, r = -cs, -sn, -r
    return cs, sn, r


def _dlaev2(a, b, c):
    sm, df = a + c, a - c
    adf, tb = abs(df), b + b
    ab = abs(tb)
    acmx, acmn = (a, c) if abs(a) > abs(c) else (c, a)
    if adf > ab:
        rt = adf * math.sqrt(1.0 + (ab / adf) ** 2)
    elif adf < ab:
        rt = ab * math.sqrt(1.0 + (adf / ab) ** 2)
    else:
        rt = ab * math.sqrt(2.0)
    if sm < 0.0:
        rt1, sgn1 = 0.5 * (sm - rt), -1
        rt2 = (acmx / rt1) * acmn - (b / rt1) * b
    elif sm > 0.0:
        rt1, sgn1 = 0.5 * (sm + rt), 1
        rt2 = (acmx / rt1) * acmn - (b / rt1) * b
    else:
        rt1, rt2, sgn1 = 0.5 * rt, -0.5 * rt, 1
    if df >= 0.0:
        cs, sgn2 = df + rt, 1
    else:
        cs, sgn2 = df - rt, -1
    if abs(cs) > ab:
        ct = -tb / cs
        sn1 = 1.0 / math.sqrt(1.0 + ct * ct)
        cs1 = ct * sn1
    elif ab == 0.0:
        cs1, sn1 = 1.0, 0.0
    else:
        tn = -cs / tb
        cs1 = 1.0 / math.sqrt(1.0 + tn * tn)
        sn1 = tn * cs1
    if sgn1 == sgn2:
        cs1, sn1 = -sn1, cs1
    return rt1, rt2, cs1, sn1


def _zlasr_rvb(Z, c, s, j0, mm, forward):
    """ZLASR('R', 'V', 'B'/'F') on columns j0 .. j0+mm-1 of Z with rotations c, s."""
    order = range(mm - 1) if forward else range(mm - 2, -1, -1)
    for j in order:
        ct, st = c[j], s[j]
        if ct != 1.0 or st != 0.0:
            t = Z[:, j0 + j + 1].copy()
            Z[:, j0 + j + 1] = ct * t - st * Z[:, j0 + j]
            Z[:, j0 + j] = st * t + ct * Z[:, j0 + j]


def zheev_lapack(A: np.ndarray, lartg: str = "new"):
    """ZHEEV(jobz='V', uplo='U') of the Hermitian A (upper triangle read): eigenvalues
    ascending and the eigenvectors as the reference LAPACK computes them."""
    n = A.shape[0]
    a = np.triu(np.asarray(A, dtype=np.complex128)).copy()
    if n == 0:
        return np.zeros(0), np.zeros((0, 0), np.complex128)
    if n == 1:
        return np.array([a[0, 0].real]), np.ones((1, 1), np.complex128)
    d = np.zeros(n)
    e = np.zeros(n - 1)
    tau = np.zeros(n - 1, np.complex128)
    # ZHETD2, uplo 'U' (0-based: reflector i annihilates a[0:i-1, i+1])
    a[n - 1, n - 1] = a[n - 1, n - 1].real

    def herm(k):   # the Hermitian matrix held in the upper triangle of a[0:k, 0:k]
        u = np.triu(a[:k, :k], 1)
        return u + u.conj().T + np.diag(a[:k, :k].diagonal().real)

    for i in range(n - 2, -1, -1):
        alpha = a[i, i + 1]
        x = a[:i, i + 1]
        xnorm = float(np.linalg.norm(x)) if i > 0 else 0.0
        alphr, alphi = alpha.real, alpha.imag
        if xnorm == 0.0 and alphi == 0.0:
            taui = 0.0 + 0.0j
        else:
            beta = -math.copysign(math.sqrt(alphr * alphr + alphi * alphi + xnorm * xnorm), alphr)
            taui = complex((beta - alphr) / beta, -alphi / beta)
            scal = 1.0 / (alpha - beta)
            a[:i, i + 1] = x * scal
            alpha = beta
        e[i] = alpha.real
        if taui != 0:
            a[i, i + 1] = 1.0
            v = a[:i + 1, i + 1].copy()
            t = taui * (herm(i + 1) @ v)
            al = -0.5 * taui * np.vdot(t, v)
            t = t + al * v
            upd = np.outer(v, t.conj()) + np.outer(t, v.conj())
            a[:i + 1, :i + 1] -= np.triu(upd)
            for q in range(i + 1):
                a[q, q] = a[q, q].real
        else:
            a[i, i] = a[i, i].real
        a[i, i + 1] = e[i]
        d[i + 1] = a[i + 1, i + 1].real
        tau[i] = taui
    d[0] = a[0, 0].real
    # ZUNGTR, uplo 'U': shift the reflector vectors one column left, then ZUNG2L
    q = np.zeros((n, n), np.complex128)
    for j in range(n - 1):
        q[:j, j] = a[:j, j + 1]
    q[n - 1, n - 1] = 1.0
    m = n - 1
    for i in range(m):        # ZUNG2L(m, m, m): ii = i
        q[i, i] = 1.0
        if i > 0:
            v = q[:i + 1, i].copy()
            C = q[:i + 1, :i]
            w = C.conj().T @ v
            q[:i + 1, :i] = C - tau[i] * np.outer(v, w.conj())
            q[:i, i] = -tau[i] * q[:i, i]
        q[i, i] = 1.0 - tau[i]
        q[i + 1:m, i] = 0.0
    Z = q
    # ZSTEQR, compz 'V'
    eps2 = _EPS * _EPS
    nmaxit, jtot = 30 * n, 0
    l1 = 0
    while l1 < n:
        if l1 > 0:
            e[l1 - 1] = 0.0
        msplit = n - 1
        for mm_ in range(l1, n - 1):
            tst = abs(e[mm_])
            if tst == 0.0:
                msplit = mm_
                break
            if tst <= math.sqrt(abs(d[mm_])) * math.sqrt(abs(d[mm_ + 1])) * _EPS:
                e[mm_] = 0.0
                msplit = mm_
                break
        l, lend = l1, msplit
        lsv, lendsv = l, lend
        l1 = msplit + 1
        if lend == l:
            continue
        anorm = max(np.abs(d[l:lend + 1]).max(), np.abs(e[l:lend]).max() if lend > l else 0.0)
        if anorm == 0.0:
            continue
        if abs(d[lend]) < abs(d[l]):
            lend, l = lsv, lendsv
        if lend > l:   # QL
            while True:
                mq = lend
                for mm_ in range(l, lend):
                    if abs(e[mm_]) ** 2 <= (eps2 * abs(d[mm_])) * abs(d[mm_ + 1]) + _SAFMIN:
                        mq = mm_
                        break
                if mq < lend:
                    e[mq] = 0.0
                p = d[l]
                if mq == l:
                    d[l] = p
                    l += 1
                    if l <= lend:
                        continue
                    break
                if mq == l + 1:
                    rt1, rt2, c, s = _dlaev2(d[l], e[l], d[l + 1])
                    _zlasr_rvb(Z, [c], [s], l, 2, forward=False)
                    d[l], d[l + 1], e[l] = rt1, rt2, 0.0
                    l += 2
                    if l <= lend:
                        continue
                    break
                if jtot == nmaxit:
                    break
                jtot += 1
                g = (d[l + 1] - p) / (2.0 * e[l])
                r = _dlapy2(g, 1.0)
                g = d[mq] - p + (e[l] / (g + math.copysign(r, g)))
                s, c, p = 1.0, 1.0, 0.0
                cw, sw = np.zeros(mq - l), np.zeros(mq - l)
                for i in range(mq - 1, l - 1, -1):
                    f = s * e[i]
                    b = c * e[i]
                    c, s, r = _dlartg(g, f, lartg)
                    if i != mq - 1:
                        e[i + 1] = r
                    g = d[i + 1] - p
                    r = (d[i] - g) * s + 2.0 * c * b
                    p = s * r
                    d[i + 1] = g + p
                    g = c * r - b
                    cw[i - l], sw[i - l] = c, -s
                _zlasr_rvb(Z, cw, sw, l, mq - l + 1, forward=False)
                d[l] -= p
                e[l] = g
        else:          # QR
            while True:
                mq = lend
                for mm_ in range(l, lend, -1):
                    if abs(e[mm_ - 1]) ** 2 <= (eps2 * abs(d[mm_])) * abs(d[mm_ - 1]) + _SAFMIN:
                        mq = mm_
                        break
                if mq > lend:
                    e[mq - 1] = 0.0
                p = d[l]
                if mq == l:
                    d[l] = p
                    l -= 1
                    if l >= lend:
                        continue
                    break
                if mq == l - 1:
                    rt1, rt2, c, s = _dlaev2(d[l - 1], e[l - 1], d[l])
                    _zlasr_rvb(Z, [c], [s], l - 1, 2, forward=True)
                    d[l - 1], d[l], e[l - 1] = rt1, rt2, 0.0
                    l -= 2
                    if l >= lend:
                        continue
                    break
                if jtot == nmaxit:
                    break
                jtot += 1
                g = (d[l - 1] - p) / (2.0 * e[l - 1])
                r = _dlapy2(g, 1.0)
                g = d[mq] - p + (e[l - 1] / (g + math.copysign(r, g)))
                s, c, p = 1.0, 1.0, 0.0
                cw, sw = np.zeros(l - mq), np.zeros(l - mq)
                for i in range(mq, l):
                    f = s * e[i]
                    b = c * e[i]
                    c, s, r = _dlartg(g, f, lartg)
                    if i != mq:
                        e[i - 1] = r
                    g = d[i] - p
                    r = (d[i + 1] - g) * s + 2.0 * c * b
                    p = s * r
                    d[i] = g + p
                    g = c * r - b
                    cw[i - mq], sw[i - mq] = c, s
                _zlasr_rvb(Z, cw, sw, mq, l - mq + 1, forward=True)
                d[l] -= p
                e[l - 1] = g
        if jtot >= nmaxit:
            raise ValueError("ZSTEQR: no convergence")
    # selection sort, swapping eigenvector columns
    for ii in range(1, n):
        i = ii - 1
        k, p = i, d[i]
        for j in range(ii, n):
            if d[j] < p:
                k, p = j, d[j]
        if k != i:
            d[k], d[i] = d[i], p
            Z[:, [i, k]] = Z[:, [k, i]]
    return d, Z


# ======================================================================================
# e0test: the CASCI energy of the selected root from its 1- and 2-RDM
# ======================================================================================
def e0test(s: System) -> Dict[str, complex]:
    """e0test (e0test.F90:4-272), run by r4dcasci after the CASCI (r4dcasci.F90:89): the
    HF-like energy of the lowest ninact + nelec spinors and the selected root's energy split
    into inactive one-electron (1), inactive two-electron (2), active one-electron with the
    inactive mean field (3) and active two-electron (4) parts, against eigen - ecore."""
    ni, na = s.ninact, s.nact
    ints = Integrals(s)
    g = ints.occ_block()                       # (pq|rs), nmoc^4
    dets = enumerate_dets(s)
    H = casmat(s, dets, g)
    w, v = heev_upper(H)
    iroot = s.selectroot - 1
    c = v[:, iroot]
    rd = RDM(FullSpace(s, dets), c, order=2)
    h = s.h
    out: Dict[str, complex] = {}
    nocc = ni + s.nelec
    out["energyHF1"] = complex(np.sum(np.diag(h)[:nocc]))
    e = 0.0 + 0.0j
    for i in range(nocc):
        for j in range(i, nocc):
            e += g[i, i, j, j] - g[i, j, j, i]
    e *= 0.5
    out["energyHF2"] = e + np.conj(e)
    out["energy1"] = complex(np.sum(np.diag(h)[:ni]))
    e = 0.0 + 0.0j
    for i in range(ni):
        for j in range(i, ni):
            e += g[i, i, j, j] - g[i, j, j, i]
    e *= 0.5
    out["energy2"] = e + np.conj(e)
    e = 0.0 + 0.0j
    for i in range(ni, ni + na):
        for j in range(i, ni + na):
            one = h[i, j] + sum(g[i, j, k, k] - g[i, k, k, j] for k in range(ni))
            if i == j:
                one *= 0.5
            e += one * rd.D1[i - ni, j - ni]
    out["energy3"] = e + np.conj(e)
    ga = g[ni:ni + na, ni:ni + na, ni:ni + na, ni:ni + na]
    e4 = np.einsum("ijkl,ijkl->", ga, rd.D2)
    e4 -= np.einsum("ijjl,il->", ga, rd.D1)
    out["energy4"] = 0.5 * e4
    out["t_energy"] = out["energy1"] + out["energy2"] + out["energy3"] + out["energy4"]
    out["eigen_minus_ecore"] = complex(w[iroot])
    out["error"] = out["eigen_minus_ecore"] - out["t_energy"]
    return out

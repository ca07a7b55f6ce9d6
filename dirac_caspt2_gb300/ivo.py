"""Improved virtual orbitals: the r4divo program (r4divo.F90:4-114) on the GPU library.

A run directory holds the IVO input (``active.ivo.inp``), MRCONEE, MDCINT(+MDCINXXXX*) and
DFPCMO.  The driver
  1. reads MRCONEE and MDCINT with the library's C++ readers and builds the MDCINTNEW stream
     and the integral classes on the device (create_newmdcint + readint2_casci);
  2. checks the virtual MO counts of DFPCMO against the input per irrep
     (module_ivo_consistency_check.F90:7-145);
  3. builds and diagonalises the IVO Fock matrix on the device (dcg_ivo: fockivo.F90:44-215);
  4. rotates the DFPCMO coefficients of each block's virtual MOs by its eigenvectors and
     writes DFPCMONEW (fockivo.F90:216-346; only the real part is written back, as there).
"""
from __future__ import annotations

import dataclasses
import os
from typing import Dict, Optional

import numpy as np

from . import api, dirac_io

__all__ = ["IvoResult", "check_consistency", "rotate_dfpcmo", "run_ivo"]


@dataclasses.dataclass
class IvoResult:
    eigenvalues: Dict[int, np.ndarray]   # per diagonalised irrep, ascending
    numh: int                            # HOMO spinors the Fock matrix removes an electron from
    dfpcmo_new: dirac_io.Dfpcmo
    path: Optional[str]


def _virtual_range(d: dirac_io.Dfpcmo, g: int, occ, vcut):
    """1-based first and last MO of group g's virtual MOs in DFPCMO."""
    mo = [p + e for p, e in zip(d.positronic, d.electronic)]
    base = 0 if g == 0 else mo[0]
    return base + d.positronic[g] + occ[g] + 1, base + mo[g] - vcut[g]


def check_consistency(d: dirac_io.Dfpcmo, inp: dirac_io.ActiveInput, irpamo: np.ndarray, nsymrpa: int) -> None:
    """module_ivo_consistency_check.F90:100-141: per fermion-irrep group and every second
    irrep, the virtual MOs of DFPCMO (by |supersymmetry|, all of them when the whole
    supersymmetry list is zero) and of the input (by irrep) must agree in number."""
    lo_in, hi_in = inp.ninact + inp.nact, inp.ninact + inp.nact + inp.nsec
    for g in range(d.nfsym):
        lo, hi = _virtual_range(d, g, inp.occ_mo_num, inp.vcut_mo_num)
        s0, s1 = (1, nsymrpa // 2) if g == 0 else (nsymrpa // 2 + 1, nsymrpa)
        for isym in range(s0, s1 + 1, 2):
            isup = isym if g == 0 else isym - nsymrpa // 2
            if np.all(d.supersym == 0):
                nv_d = hi - lo + 1
            else:
                nv_d = int(np.count_nonzero(np.abs(d.supersym[lo - 1:hi]) == isup))
            nv_i = int(np.count_nonzero(np.asarray(irpamo[lo_in:hi_in]) == isym))
            if nv_i != nv_d:
                raise ValueError(f"IVO: irrep {isym} has {nv_d} virtual MOs in DFPCMO and {nv_i} in the input "
                                 "(check .nvcut/.nvcutg/.nvcutu)")


def rotate_dfpcmo(d: dirac_io.Dfpcmo, inp: dirac_io.ActiveInput, U: np.ndarray, block_isym: np.ndarray,
                  nsymrpa: int) -> dirac_io.Dfpcmo:
    """fockivo.F90:216-285: for each block, the coefficient columns of its virtual MOs times
    the block's eigenvectors; the real part is stored back."""
    coef = d.coef.copy()
    mo = [p + e for p, e in zip(d.positronic, d.electronic)]
    for g in range(d.nfsym):
        nao = d.basis_ao[g]
        base = (0 if g == 0 else d.basis_all[0]) + (d.positronic[g] + inp.occ_mo_num[g]) * nao
        nvirt = d.electronic[g] - inp.occ_mo_num[g] - inp.vcut_mo_num[g]
        itrfmo = coef[base:base + nvirt * nao].reshape(nvirt, nao).T.astype(np.complex128)
        mo_off = (0 if g == 0 else mo[0]) + d.positronic[g] + inp.occ_mo_num[g]
        lo, hi = _virtual_range(d, g, inp.occ_mo_num, inp.vcut_mo_num)
        s0, s1 = (1, nsymrpa // 2) if g == 0 else (nsymrpa // 2 + 1, nsymrpa)
        for isym in range(s0, s1 + 1, 2):
            sec = np.flatnonzero(block_isym == isym)
            if len(sec) == 0:
                continue
            isup = isym if g == 0 else isym - nsymrpa // 2
            sup = d.supersym[lo - 1:hi]
            mos = np.arange(lo, hi + 1)
            dmosym = mos if np.all(sup == 0) else mos[np.abs(sup) == isup]
            if len(dmosym) != len(sec):
                raise ValueError(f"IVO: irrep {isym}: {len(dmosym)} DFPCMO MOs for {len(sec)} block spinors")
            cols = dmosym - mo_off - 1
            itrfmo[:, cols] = itrfmo[:, cols] @ U[np.ix_(sec, sec)]
        coef[base:base + nvirt * nao] = itrfmo.real.T.reshape(-1)
    return dataclasses.replace(d, coef=coef)


def run_ivo(directory: str, input_name: str = "active.ivo.inp", out_path: Optional[str] = None,
            session: Optional[api.Caspt2Session] = None, device: int = 0) -> IvoResult:
    """The IVO program on one run directory; writes ``out_path`` (default DFPCMONEW in the
    directory) and returns the IVO eigenvalues."""
    inp = dirac_io.read_active_inp(os.path.join(directory, input_name))
    d = dirac_io.read_dfpcmo(os.path.join(directory, "DFPCMO"), inp.diracver >= 21)
    own = session is None
    ses = session or api.Caspt2Session(device)
    try:
        with api.NativeFiles(directory, inp) as nf:
            m = nf.mrconee()
            check_consistency(d, inp, m.irpamo, m.nsymrpa)
            ses.set_system_mdcint(nf.system_input(), nf)
            eps, U, bsym, numh = ses.ivo(d.nfsym, m.mo_energy, inp.nhomo)
    finally:
        if own:
            ses.close()
    new = rotate_dfpcmo(d, inp, U, bsym, m.nsymrpa)
    path = out_path if out_path is not None else os.path.join(directory, "DFPCMONEW")
    if path:
        dirac_io.write_dfpcmo(path, new)
    evals = {int(s): eps[bsym == s] for s in np.unique(bsym) if s > 0}
    return IvoResult(eigenvalues=evals, numh=numh, dfpcmo_new=new, path=path or None)

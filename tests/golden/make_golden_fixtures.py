"""Regenerate the golden fixtures from the reference's runnable test cases.

For each case directory of the reference's ``test/dev`` tree that ships its MDCINT files,
this reads ``active.inp``, ``MRCONEE`` and ``MDCINT*`` with the package's readers
(restatements of read_mrconee / create_newmdcint) and stores the resulting system in
``<case>.npz`` together with the energies printed in ``reference.<case>.out``:
the CASCI total energy of the selected root, the per-subspace ``e2X`` and ``sumc2,X``, the
per-irrep ``e2X(isym)`` lines (``ref_e2_sym``, (8, nsymrpa), NaN where the reference prints
none), the total CASPT2 energy and the e0test terms (energyHF(1..2), energy 1..4).  For every
case it also stores the raw MDCINT records (``<case>_mdcint_raw.npz``), the input of the MDCINT
canonicalisation, together with the case's MRCONEE bytes and active.inp text, so that a test
can rewrite the run directory (for instance with MDCINT in the complex record format) and read
it back through the library's own readers.

For the IVO cases (``ivo_*.npz``): the system read with ``active.ivo.inp``, the MDCINTNEW
records IVO reads (two secondary and two active indices: the (ab|kk) and (ak|kb) classes of
fockivo.F90:56-85), the orbital energies, the IVO keywords, the DFPCMO text and the
coefficients of the reference's ``reference.DFPCMONEW``.

Usage:  python tests/golden/make_golden_fixtures.py /path/to/reference/test/dev
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from dirac_caspt2_gb300 import dirac_io  # noqa: E402

CASES = ["c2_h2o_dev", "check_minelecras3_dev", "ninact_0_h2_dev", "mdcint_scheme_6_dirac23_c32h_n2_dev"]
RAW_CASES = CASES


def parse_e0test(path: str):
    """The e0test block (e0test.F90:85-270): energyHF(1), energyHF(2), energy 1..4 (real parts
    of the printed complex numbers), NaN where absent."""
    keys = [r"energyHF\(1\)", r"energyHF\(2\)", "energy 1 =", "energy 2 =", "energy 3 =", "energy 4 ="]
    out = [np.nan] * len(keys)
    for ln in open(path, errors="replace").read().splitlines():
        for q, k in enumerate(keys):
            m = re.match(r"^\s*" + k + r"\s*\(\s*([-+0-9.Ee]+)\s*,", ln)
            if m and np.isnan(out[q]):
                out[q] = float(m.group(1))
    return np.array(out)


def parse_e2_sym(path: str, nsym: int):
    """The e2X(isym) lines of solve_A..G_subspace (e.g. solve_A_subspace.F90:262) as an
    (8, nsym) array, NaN where nothing is printed."""
    out = np.full((8, nsym), np.nan)
    for ln in open(path, errors="replace").read().splitlines():
        m = re.match(r"^\s*e2([a-h])\(\s*(\d+)\)\s*=\s*([-+0-9.Ee]+)\s*a\.u\.", ln)
        if m:
            out["abcdefgh".index(m.group(1)), int(m.group(2)) - 1] = float(m.group(3))
    return out


def parse_output(path: str, selectroot: int):
    txt = open(path, errors="replace").read().splitlines()
    e2, sc2 = {}, {}
    casci = None
    total = None
    for ln in txt:
        m = re.match(r"^\s*e2([a-h])\s*=\s*([-+0-9.Ee]+)\s*a\.u\.", ln)
        if m:
            e2[m.group(1).upper()] = float(m.group(2))
        m = re.match(r"^\s*sumc2,([a-h])\s*=\s*([-+0-9.Ee]+)", ln)
        if m:
            sc2[m.group(1).upper()] = float(m.group(2))
        m = re.match(r"^CASCI Total Energy ROOT(\d+)\s+([-+0-9.Ee]+)\s+a\.u\.", ln)
        if m and int(m.group(1)) == selectroot and casci is None:
            casci = float(m.group(2))
        m = re.match(r"^\s*Total energy is\s+([-+0-9.Ee]+)\s+a\.u\.", ln)
        if m:
            total = float(m.group(1))
    return casci, e2, sc2, total


def main(devdir: str):
    for case in CASES:
        d = os.path.join(devdir, case)
        inp = dirac_io.read_active_inp(os.path.join(d, "active.inp"))
        mrc = dirac_io.read_mrconee(os.path.join(d, "MRCONEE"), inp)
        new = dirac_io.read_mdcint_new(d, mrc, inp)
        ts, sr = inp.ciroots[0]
        casci, e2, sc2, total = parse_output(os.path.join(d, f"reference.{case}.out"), sr)
        out = dict(ninact=inp.ninact, nact=inp.nact, nsec=inp.nsec, nelec=inp.nelec, nmo=mrc.nmo,
                   nsymrpa=mrc.nsymrpa, multb=mrc.multb.astype(np.int32), irpamo=mrc.irpamo.astype(np.int32),
                   h_re=mrc.h.real, h_im=mrc.h.imag, ecore=mrc.ecore,
                   rec_idx=new.idx.astype(np.int16), rec_re=new.val.real, realonly=new.realonly,
                   totsym=ts, selectroot=sr, eshift=inp.eshift,
                   ras=np.array([len(inp.ras1), len(inp.ras2), len(inp.ras3)], dtype=np.int32),
                   ras1_max_hole=inp.ras1_max_hole, ras3_max_elec=inp.ras3_max_elec,
                   min_hole_ras1=inp.min_hole_ras1, min_elec_ras3=inp.min_elec_ras3,
                   ref_casci=casci, ref_total=total,
                   ref_e2=np.array([e2.get(k, np.nan) for k in "ABCDEFGH"]),
                   ref_sumc2=np.array([sc2.get(k, np.nan) for k in "ABCDEFGH"]),
                   ref_e2_sym=parse_e2_sym(os.path.join(d, f"reference.{case}.out"), mrc.nsymrpa),
                   ref_e0test=parse_e0test(os.path.join(d, f"reference.{case}.out")))
        if not new.realonly:
            out["rec_im"] = new.val.imag
        np.savez_compressed(os.path.join(HERE, f"{case}.npz"), **out)
        print(case, "records", len(new), "total", total)
        if case in RAW_CASES:   # the MDCINT records themselves, for the device canonicalisation
            raw = dirac_io.read_mdcint_raw(d, mrc, inp)
            np.savez_compressed(os.path.join(HERE, f"{case}_mdcint_raw.npz"), rec_ikr=raw.rec_ikr,
                                rec_jkr=raw.rec_jkr, rec_off=raw.rec_off, indk=raw.indk, indl=raw.indl, re=raw.re,
                                im=raw.im, kr=raw.kr, nmo=raw.nmo, dirac_to_cas=raw.dirac_to_cas,
                                scheme=raw.scheme, realonly=raw.realonly,
                                mrconee=np.frombuffer(open(os.path.join(d, "MRCONEE"), "rb").read(), np.uint8),
                                active_inp=open(os.path.join(d, "active.inp")).read(),
                                dirac_32bit=mrc.dirac_32bit)
            print(case, "raw entries", len(raw.re))


IVO_CASES = ["ivo_c32h_ar_with_kappa_dev", "ivo_c32h_n2_dev_dirac19", "ivo_c32h_n2_dev_dirac22"]


def main_ivo(devdir: str):
    for case in IVO_CASES:
        d = os.path.join(devdir, case)
        inp = dirac_io.read_active_inp(os.path.join(d, "active.ivo.inp"))
        mrc = dirac_io.read_mrconee(os.path.join(d, "MRCONEE"), inp)
        new = dirac_io.read_mdcint_new(d, mrc, inp)
        ni, na, ns = inp.ninact, inp.nact, inp.nsec
        g = new.idx.astype(np.int64) - 1
        sp = np.where(g < ni, 1, np.where(g < ni + na, 2, np.where(g < ni + na + ns, 3, 4)))
        keep = ((sp == 3).sum(axis=1) == 2) & ((sp == 2).sum(axis=1) == 2)
        ref = dirac_io.read_dfpcmo(os.path.join(d, "reference.DFPCMONEW"), inp.diracver >= 21)
        out = dict(ninact=ni, nact=na, nsec=ns, nelec=inp.nelec, nmo=mrc.nmo, nsymrpa=mrc.nsymrpa,
                   multb=mrc.multb.astype(np.int32), irpamo=mrc.irpamo.astype(np.int32), h_re=mrc.h.real,
                   h_im=mrc.h.imag, ecore=mrc.ecore, mo_energy=mrc.mo_energy, realonly=new.realonly,
                   rec_idx=new.idx[keep].astype(np.int16), rec_re=new.val.real[keep], diracver=inp.diracver,
                   nhomo=inp.nhomo, occ_mo_num=np.array(inp.occ_mo_num, np.int32),
                   vcut_mo_num=np.array(inp.vcut_mo_num, np.int32), inversion=inp.inversion,
                   dfpcmo_text=np.frombuffer(open(os.path.join(d, "DFPCMO"), "rb").read(), np.uint8),
                   ref_coef=ref.coef)
        if not new.realonly:
            out["rec_im"] = new.val.imag[keep]
        np.savez_compressed(os.path.join(HERE, f"{case}.npz"), **out)
        print(case, "records", int(keep.sum()), "of", len(new))


if __name__ == "__main__":
    top = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/test/dev"
    main(top)
    main_ivo(top)

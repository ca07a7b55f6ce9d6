"""IVO (r4divo / fockivo): the oracle pinned on the reference's three runnable IVO cases
(their reference.DFPCMONEW coefficients at the reference test's own tolerance, 1e-13), the
restated LAPACK ZHEEV, the DFPCMO reader/writer, the IVO input keywords and the host-side
rotation and consistency check of the driver.  CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR

IVO_CASES = ["ivo_c32h_ar_with_kappa_dev", "ivo_c32h_n2_dev_dirac19", "ivo_c32h_n2_dev_dirac22"]


def load_ivo_fixture(case):
    """(oracle System, mo_energy, ActiveInput-like keywords, Dfpcmo, reference coefficients)."""
    from dirac_caspt2_gb300 import dirac_io
    from oracle import caspt2_oracle as O
    z = np.load(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    val = z["rec_re"] + (1j * z["rec_im"] if "rec_im" in z.files else 0.0)
    s = O.System(ninact=int(z["ninact"]), nact=int(z["nact"]), nsec=int(z["nsec"]), nelec=int(z["nelec"]),
                 nmo=int(z["nmo"]), nsymrpa=int(z["nsymrpa"]), multb=z["multb"].astype(np.int64),
                 irpamo=z["irpamo"].astype(np.int64), h=z["h_re"] + 1j * z["h_im"], ecore=float(z["ecore"]),
                 rec_idx=z["rec_idx"].astype(np.int32), rec_val=np.asarray(val, np.complex128),
                 realonly=bool(z["realonly"]))
    inp = dirac_io.ActiveInput(ninact=s.ninact, nact=s.nact, nsec=s.nsec, nelec=s.nelec, ciroots=[(33, 1)],
                               diracver=int(z["diracver"]), nhomo=int(z["nhomo"]),
                               occ_mo_num=tuple(int(x) for x in z["occ_mo_num"]),
                               vcut_mo_num=tuple(int(x) for x in z["vcut_mo_num"]), inversion=bool(z["inversion"]))
    text = bytes(z["dfpcmo_text"]).decode()
    d = _read_dfpcmo_text(text, inp.diracver >= 21)
    return s, z["mo_energy"], inp, d, z["ref_coef"], text


def _read_dfpcmo_text(text, new_format):
    import tempfile
    from dirac_caspt2_gb300 import dirac_io
    with tempfile.NamedTemporaryFile("w", suffix=".dfpcmo", delete=False) as f:
        f.write(text)
        name = f.name
    try:
        return dirac_io.read_dfpcmo(name, new_format)
    finally:
        os.unlink(name)


@pytest.mark.parametrize("case", IVO_CASES)
def test_oracle_ivo_matches_reference_dfpcmonew(case):
    from oracle import caspt2_oracle as O
    s, me, inp, d, ref, _ = load_ivo_fixture(case)
    ints = O.Integrals(s)
    coef, ev, numh = O.ivo(s, ints, me, d, inp.nhomo, inp.occ_mo_num, inp.vcut_mo_num, lartg="old")
    assert numh == 6
    assert np.abs(coef - ref).max() <= 1e-13          # the reference test's tolerance
    assert not np.array_equal(coef, d.coef)            # the virtual MOs did rotate


def test_oracle_ivo_needs_lapack39_rotation_signs():
    """The Givens generator of LAPACK >= 3.10 flips some IVO orbitals of the N2 case: the
    reference's DFPCMONEW carries the signs of the older one."""
    from oracle import caspt2_oracle as O
    s, me, inp, d, ref, _ = load_ivo_fixture("ivo_c32h_n2_dev_dirac22")
    coef, _, _ = O.ivo(s, O.Integrals(s), me, d, inp.nhomo, inp.occ_mo_num, inp.vcut_mo_num, lartg="new")
    assert np.abs(coef - ref).max() > 1.0
    assert np.abs(np.abs(coef) - np.abs(ref)).max() <= 1e-13


@pytest.mark.parametrize("n", [1, 2, 3, 7, 16, 40])
@pytest.mark.parametrize("cplx", [False, True])
def test_zheev_lapack_is_an_eigensolver(n, cplx):
    from oracle import caspt2_oracle as O
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if cplx else 0)
    A = A + A.conj().T
    for v in ("old", "new"):
        w, Z = O.zheev_lapack(np.triu(A), v)
        assert np.abs(w - np.linalg.eigvalsh(A)).max() <= 1e-12 * max(1.0, np.abs(w).max())
        assert np.abs(A @ Z - Z * w).max() <= 1e-12 * max(1.0, np.abs(w).max())
        assert np.abs(Z.conj().T @ Z - np.eye(n)).max() <= 1e-13


@pytest.mark.parametrize("case", IVO_CASES)
def test_dfpcmo_writer_reproduces_the_file(case, tmp_path):
    """Reading DFPCMO and writing it back gives the same tokens (F22.16 coefficients, E22.12
    energies, I0 integers, title lines)."""
    from dirac_caspt2_gb300 import dirac_io
    s, me, inp, d, ref, text = load_ivo_fixture(case)
    p = str(tmp_path / "out")
    dirac_io.write_dfpcmo(p, d)
    a = [ln.split() for ln in text.splitlines()]
    b = [ln.split() for ln in open(p).read().splitlines()]
    assert a == b


def test_ivo_input_keywords():
    from dirac_caspt2_gb300 import dirac_io
    a = dirac_io.read_active_inp(".ninact\n0\n.nact\n14\n.nelec\n14\n.nsec\n24\n.noccg\n3\n.noccu\n6\n"
                                 ".nvcutg\n10\n.nvcutu\n15\n.nhomo\n2\n.caspt2_ciroots\n33 1\n.diracver\n22\n"
                                 ".subprograms\nIVO\n.end\n")
    assert a.inversion and a.occ_mo_num == (3, 6) and a.vcut_mo_num == (10, 15) and a.nhomo == 2
    b = dirac_io.read_active_inp(".ninact\n0\n.nact\n10\n.nsec\n28\n.nelec\n10\n.nocc\n5\n.nvcut\n11\n"
                                 ".diracver\n22\n.end\n")
    assert not b.inversion and b.occ_mo_num == (5, 0) and b.vcut_mo_num == (11, 0)
    with pytest.raises(ValueError):
        dirac_io.read_active_inp(".ninact\n0\n.nact\n2\n.nsec\n2\n.nelec\n2\n.nocc\n1\n.noccg\n1\n"
                                 ".diracver\n22\n.end\n")


@pytest.mark.parametrize("case", IVO_CASES[:2])
def test_driver_rotation_and_consistency(case):
    """The driver's host steps: the DFPCMO rotation by per-block eigenvectors (here the
    oracle's) gives the oracle's coefficients; a DFPCMO whose virtual MO count disagrees with
    the input is refused."""
    import dataclasses
    from dirac_caspt2_gb300 import ivo
    from oracle import caspt2_oracle as O
    s, me, inp, d, ref, _ = load_ivo_fixture(case)
    ints = O.Integrals(s)
    coef, ev, numh = O.ivo(s, ints, me, d, inp.nhomo, inp.occ_mo_num, inp.vcut_mo_num, lartg="old")
    fu, _ = O.ivo_fock(s, ints, me, inp.nhomo)
    U = np.zeros((s.nsec, s.nsec), np.complex128)
    bsym = np.zeros(s.nsec, np.int32)
    for isym, sec in O.ivo_blocks(s, d.nfsym):
        if len(sec) == 0:
            continue
        fs = fu[np.ix_(sec, sec)]
        A = np.triu(fs, 1) + np.triu(fs, 1).conj().T + np.diag(fs.diagonal().real)
        w, V = O.zheev_lapack(A, "old")
        U[np.ix_(sec, sec)] = V
        bsym[sec] = isym
    ivo.check_consistency(d, inp, s.irpamo, s.nsymrpa)
    new = ivo.rotate_dfpcmo(d, inp, U, bsym, s.nsymrpa)
    assert np.array_equal(new.coef, coef)
    bad = dataclasses.replace(inp, vcut_mo_num=(inp.vcut_mo_num[0] + 2, inp.vcut_mo_num[1]))
    with pytest.raises(ValueError):
        ivo.check_consistency(d, bad, s.irpamo, s.nsymrpa)

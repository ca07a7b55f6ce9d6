"""The CPU oracle reproduces the reference's own printed energies on every runnable golden
case (per subspace and total, abs 1e-10 Eh: the reference tests' tolerance)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_CASES, GOLDEN_DIR, oracle_system

TOL = 1e-10


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_matches_reference_golden(case):
    from dirac_caspt2_gb300 import api
    from oracle import caspt2_oracle as O
    path = os.path.join(GOLDEN_DIR, f"{case}.npz")
    s = api.SystemInput.from_npz(path)
    z = np.load(path)
    r = O.run(oracle_system(s))
    assert abs(r.casci_energies[s.selectroot - 1] - float(z["ref_casci"])) < TOL
    for i, k in enumerate("ABCDEFGH"):
        ref = z["ref_e2"][i]
        if np.isnan(ref):        # subspace skipped by the reference (ninact = 0 or nsec = 0)
            assert k not in r.e2
            continue
        assert abs(r.e2[k] - ref) < TOL, (k, r.e2[k], ref)
        assert abs(r.sumc2[k] - z["ref_sumc2"][i]) < TOL, (k, r.sumc2[k], z["ref_sumc2"][i])
    assert abs(r.total_energy - float(z["ref_total"])) < TOL


E0TEST_KEYS = ("energyHF1", "energyHF2", "energy1", "energy2", "energy3", "energy4")


@pytest.mark.parametrize("case", [c for c in GOLDEN_CASES if "c32h_n2" not in c])
def test_oracle_e0test_matches_reference(case):
    """e0test's printed terms (energyHF(1..2), energy 1..4) and its error line."""
    from dirac_caspt2_gb300 import api
    from oracle import caspt2_oracle as O
    s = api.SystemInput.from_npz(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    z = np.load(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    r = O.e0test(oracle_system(s))
    got = np.array([r[k].real for k in E0TEST_KEYS])
    assert np.abs(got - z["ref_e0test"]).max() <= 1e-10
    assert abs(r["error"]) <= 1e-10


def check_e2_sym(e2_sym, ref, tol=TOL):
    """e2_sym {subspace: {isym: e2}} against the golden (8, nsym) e2X(isym) array: the same set of
    printed lines (solve_X_subspace prints a block with a kept dimension) and their values."""
    for i, k in enumerate("ABCDEFG"):
        want = {q + 1: float(v) for q, v in enumerate(ref[i]) if not np.isnan(v)}
        got = e2_sym.get(k, {})
        assert sorted(got) == sorted(want), (k, sorted(got), sorted(want))
        for q, v in want.items():
            assert abs(got[q] - v) < tol, (k, q, got[q], v)
    assert not e2_sym.get("H")


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_per_irrep_energies_match_reference(case):
    """The e2X(isym) lines every solve_A..G_subspace prints (e.g. solve_A_subspace.F90:262)."""
    from dirac_caspt2_gb300 import api
    from oracle import caspt2_oracle as O
    path = os.path.join(GOLDEN_DIR, f"{case}.npz")
    s = api.SystemInput.from_npz(path)
    r = O.run(oracle_system(s))
    check_e2_sym(r.e2_sym, np.load(path)["ref_e2_sym"])

"""RAS CASCI on the GPU: the determinant space restricted by .ras1/.ras3 (ras_det_check.F90,
search_cas_configuration.F90:91-110) and its lowest roots from the dense solver, from block
Davidson and from the oracle, on synthetic systems of 554 and 1619 RAS determinants: roots
within 1e-10 Eh of the oracle and 1e-11 Eh between the two device solvers (stated tolerances).
This is the route the 74 273-determinant RAS configuration (RAS1 8 / RAS2 10 / RAS3 8,
10 electrons) takes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [((2, 12, 8, 6), (4, 4, 4), 554), ((2, 14, 6, 6), (4, 6, 4), 1619)]


def _sys(dims, ras, realonly):
    from dirac_caspt2_gb300 import api, synth
    S = synth.make_system(synth.SynthConfig(*dims, seed=41, realonly=realonly))
    s = api.SystemInput.from_synth(S)
    s.ras = ras
    s.ras1_max_hole = 2
    s.ras3_max_elec = 2
    return s


@pytest.mark.parametrize("dims,ras,ndet", CASES)
@pytest.mark.parametrize("realonly", [False, True])
def test_ras_casci_dense_davidson_oracle(gpu_lib, dims, ras, ndet, realonly):
    from dirac_caspt2_gb300 import api
    s = _sys(dims, ras, realonly)
    out = {}
    with api.Caspt2Session(0) as ses:
        ses.set_system(s)
        for solver in ("dense", "davidson"):
            ses.set_casci_solver(solver)
            e, n = ses.casci(3)
            assert n == ndet
            out[solver] = np.asarray(e)
    assert np.abs(out["dense"] - out["davidson"]).max() <= 1e-11
    if ndet <= 600:
        from oracle import caspt2_oracle as O
        from conftest import oracle_system
        ref = O.run(oracle_system(s), subspaces="")
        assert ref.ndet == ndet
        assert np.abs(out["davidson"] - ref.casci_energies[:3]).max() <= 1e-10


@pytest.mark.parametrize("realonly", [False, True])
def test_ras_caspt2_matches_oracle(gpu_lib, realonly):
    """RASPT2 through the whole path (RAS CI space, the CI rotation by the linear solve of the
    restricted determinant list, densities, A-H) against the oracle: every e2 within 1e-9 Eh,
    the total within 1e-10 Eh."""
    from dirac_caspt2_gb300 import api, synth
    from oracle import caspt2_oracle as O
    from conftest import oracle_system
    S = synth.make_system(synth.SynthConfig(4, 8, 10, 4, seed=43, realonly=realonly))
    s = api.SystemInput.from_synth(S)
    s.ras = (2, 4, 2)
    s.ras1_max_hole = 1
    s.ras3_max_elec = 1
    with api.Caspt2Session(0) as ses:
        r = ses.solve(s)
    ref = O.run(oracle_system(s))
    assert r.ndet == ref.ndet and r.ndet < 70    # restricted below the 70 of the full space
    for k in "ABCDEFGH":
        assert abs(r.e2[k] - ref.e2[k]) <= 1e-9, k
    assert abs(r.total_energy - ref.total_energy) <= 1e-10

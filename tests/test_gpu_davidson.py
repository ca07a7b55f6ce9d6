"""The block Davidson CASCI eigensolver (dcg_set_casci_solver DAVIDSON) against the dense
Householder/divide-and-conquer solver on the same Hamiltonians: the requested roots within
1e-11 Eh, and the CASPT2 energies that depend on the selected root's vector within 1e-10 Eh
(stated tolerances).  Cases: complex and real, several roots, a root above the ground state,
the Kramers-degenerate spectrum of an odd electron count (energies only), and the
determinant count of the 20/12/300 workload (924), where AUTO picks Davidson."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_E = 1e-11
TOL_E2 = 1e-10


def _solve(sysin, solver, nroot=1):
    from dirac_caspt2_gb300 import api
    with api.Caspt2Session(0) as ses:
        ses.set_casci_solver(solver)
        ses.set_system(sysin)
        eig, ndet = ses.casci(max(nroot, sysin.selectroot))
        its = ses.casci_iterations()
        e2, sc, e0, et = ses.caspt2()
    return eig, ndet, e2, sc, e0, et, its


@pytest.mark.parametrize("ni,na,ns,ne,realonly,selectroot,nroot", [
    (4, 10, 12, 4, False, 1, 1),     # 210 determinants
    (2, 10, 8, 4, True, 1, 3),       # 210, real, three roots
    (4, 10, 10, 6, False, 3, 3),     # a root above the ground state
    (4, 12, 8, 4, False, 2, 2),      # 495
    (2, 12, 6, 6, False, 1, 1),      # 924
])
def test_davidson_matches_dense(gpu_lib, ni, na, ns, ne, realonly, selectroot, nroot):
    from dirac_caspt2_gb300 import api, synth
    S = synth.make_system(synth.SynthConfig(ni, na, ns, ne, seed=21, realonly=realonly))
    s = api.SystemInput.from_synth(S, selectroot=selectroot)
    d = _solve(s, "dense", nroot)
    v = _solve(s, "davidson", nroot)
    assert d[6] == 0 and v[6] > 0
    assert d[1] == v[1]
    assert np.abs(np.asarray(d[0]) - np.asarray(v[0])).max() <= TOL_E
    for k in "ABCDEFGH":
        assert abs(d[2][k] - v[2][k]) <= TOL_E2, k
        assert abs(d[3][k] - v[3][k]) <= TOL_E2, k
    assert abs(d[4] - v[4]) <= TOL_E2
    assert abs(d[5] - v[5]) <= TOL_E2


def test_davidson_degenerate_roots(gpu_lib):
    """Odd electron count: Kramers pairs; the Davidson block holds both members."""
    from dirac_caspt2_gb300 import api, synth
    S = synth.make_system(synth.SynthConfig(2, 10, 4, 5, seed=4))
    s = api.SystemInput.from_synth(S)
    with api.Caspt2Session(0) as ses:
        ses.set_system(s)
        ses.set_casci_solver("dense")
        ed, nd = ses.casci(4)
        ses.set_casci_solver("davidson")
        ev, nv = ses.casci(4)
    assert nd == nv == 252
    assert np.abs(ed - ev).max() <= TOL_E
    assert abs(ev[0] - ev[1]) <= TOL_E and abs(ev[2] - ev[3]) <= TOL_E


def test_auto_picks_by_size(gpu_lib):
    """AUTO: dense at 495 determinants, Davidson at 924 (the 20/12/300 CASCI) and 3003, all
    equal to the dense roots."""
    from dirac_caspt2_gb300 import api, synth
    for dims, want_dav in (((2, 12, 6, 4), False), ((2, 12, 6, 6), True), ((2, 14, 4, 8), True)):
        S = synth.make_system(synth.SynthConfig(*dims, seed=8))
        s = api.SystemInput.from_synth(S)
        with api.Caspt2Session(0) as ses:
            ses.set_system(s)
            ses.set_casci_solver("dense")
            ed, _ = ses.casci(2)
            ses.set_casci_solver("auto")
            ea, _ = ses.casci(2)
            assert (ses.casci_iterations() > 0) == want_dav
        assert np.abs(ed - ea).max() <= TOL_E


def test_solver_option_rejects_bad_values(gpu_lib):
    from dirac_caspt2_gb300 import api
    lib = api.load_library()
    with api.Caspt2Session(0) as ses:
        assert lib.dcg_set_casci_solver(ses.h, 3) == -1
        assert lib.dcg_set_casci_solver(ses.h, -1) == -1

"""The CASCI hand-off of the boundary against the oracle: the determinant list dcg_casci works
in (dcg_casci_determinants) is the reference's dict_cas_idx, bit for bit and in the same
order (search_cas_configuration.F90:33-56: ascending bit strings through Gosper's hack, RAS
and totsym filtered), and the CI coefficients cir/cii dcg_casci returns, the content of
CIDATA_sym<n> (casci.F90:118-160), equal the oracle's ZHEEV eigenvectors up to one global
phase within 1e-10 per coefficient.  Cases: the four reference goldens (point-group symmetry,
RAS, ninact = 0), synthetic complex and real CAS spaces on the dense solver and on Davidson
(924 determinants), and a RAS space."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from conftest import GOLDEN_CASES, GOLDEN_DIR, oracle_system

TOL = 1e-10


def _oracle_casci(s):
    from oracle import caspt2_oracle as O
    sysm = oracle_system(s)
    dets = O.enumerate_dets(sysm)
    H = O.casmat(sysm, dets, O.Integrals(sysm).occ_block())
    w, v = O.heev_upper(H)
    return np.array(dets, np.int64), w, v


def _check(s, solver="auto"):
    from dirac_caspt2_gb300 import api
    dets_ref, w, v = _oracle_casci(s)
    root = s.selectroot - 1
    if len(w) > root + 1:   # a degenerate root has no unique vector to compare
        assert w[root + 1] - w[root] > 1e-6
    with api.Caspt2Session(0) as ses:
        ses.set_system(s)
        ses.set_casci_solver(solver)
        eig, ndet, C = ses.casci(s.selectroot, want_ci=True)
        dets = ses.casci_determinants(ndet)
    assert ndet == len(dets_ref)
    assert np.array_equal(dets, dets_ref)
    c, r = C[:, root], v[:, root]
    ph = np.vdot(r, c)                      # c = e^{i phi} r
    assert abs(abs(ph) - 1.0) < TOL
    assert np.abs(c - ph * r).max() < TOL
    assert abs(eig[root] - (w[root] + s.ecore)) < TOL


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_ci_vectors_golden(gpu_lib, case):
    from dirac_caspt2_gb300 import api
    _check(api.SystemInput.from_npz(os.path.join(GOLDEN_DIR, f"{case}.npz")))


@pytest.mark.parametrize("dims,realonly,solver", [
    ((4, 6, 8, 2), False, "dense"),
    ((8, 6, 40, 4), False, "dense"),
    ((4, 8, 8, 4), True, "dense"),
    ((2, 12, 4, 6), False, "davidson"),   # 924 determinants, the AUTO route at this size
])
def test_ci_vectors_synthetic(gpu_lib, dims, realonly, solver):
    from dirac_caspt2_gb300 import api, synth
    S = synth.make_system(synth.SynthConfig(*dims, seed=5, realonly=realonly))
    _check(api.SystemInput.from_synth(S), solver)


@pytest.mark.parametrize("realonly", [False, True])
def test_ci_vectors_ras(gpu_lib, realonly):
    from dirac_caspt2_gb300 import api, synth
    S = synth.make_system(synth.SynthConfig(2, 12, 8, 6, seed=41, realonly=realonly))
    s = api.SystemInput.from_synth(S)
    s.ras = (4, 4, 4)
    s.ras1_max_hole = 2
    s.ras3_max_elec = 2
    _check(s)

"""The dense density tensors of the oracle equal the reference's determinant loops
(density_matrix.F90:3-247) element by element, and the CASCI matrix is Hermitian."""
import numpy as np
import pytest


def _small_system(seed=4, ras=False):
    from dirac_caspt2_gb300 import synth
    from oracle import caspt2_oracle as O
    S = synth.make_system(synth.SynthConfig(2, 4, 4, 2, seed=seed))
    kw = {}
    if ras:
        kw = dict(ras1=(0, 1), ras2=(2,), ras3=(3,), ras1_max_hole=1, ras3_max_elec=1)
    return O.System(ninact=2, nact=4, nsec=4, nelec=2, nmo=S.nmo, nsymrpa=1, multb=S.multb, irpamo=S.irpamo,
                    h=S.h, ecore=S.ecore, rec_idx=S.rec_idx, rec_val=S.rec_val, realonly=False, **kw)


@pytest.mark.parametrize("ras", [False, True])
def test_rdm_tensors_equal_literal_loops(ras):
    from oracle import caspt2_oracle as O
    s = _small_system(ras=ras)
    dets = O.enumerate_dets(s)
    rng = np.random.default_rng(0)
    c = rng.normal(size=len(dets)) + 1j * rng.normal(size=len(dets))
    c /= np.linalg.norm(c)
    fs = O.FullSpace(s, dets)
    eps = rng.uniform(-1, 1, s.nact)
    rd = O.RDM(fs, c, eps_act=eps, order=3)
    na = s.nact
    for _ in range(40):
        a, b, cc, d, e, f = rng.integers(0, na, 6)
        lit = O.density_literal([(a, b), (cc, d), (e, f)], dets, c, na)
        assert abs(rd.D3[a, b, cc, d, e, f] - lit) < 1e-14
        lit2 = O.density_literal([(a, b), (cc, d)], dets, c, na)
        assert abs(rd.D2[a, b, cc, d] - lit2) < 1e-14
        lit3 = sum(eps[w] * O.density_literal([(a, b), (cc, d), (e, f), (w, w)], dets, c, na) for w in range(na))
        assert abs(rd.T3[a, b, cc, d, e, f] - lit3) < 1e-14


def test_casci_matrix_hermitian_and_oracle_deterministic():
    from oracle import caspt2_oracle as O
    s = _small_system()
    ints = O.Integrals(s)
    dets = O.enumerate_dets(s)
    H = O.casmat(s, dets, ints.occ_block())
    assert np.abs(H - H.conj().T).max() < 1e-14
    r1, r2 = O.run(s), O.run(s)
    assert r1.total_energy == r2.total_energy

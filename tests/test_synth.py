"""Synthetic generator: Hermitian, time-reversal-symmetric operators and a canonical record
set whose 16-partner expansion reproduces the dense two-electron tensor."""
import itertools

import numpy as np
import pytest


def _tr_sign(n):
    x = np.arange(n) + 1
    return np.where((x[:, None] + x[None, :]) % 2 == 0, 1.0, -1.0)


@pytest.mark.parametrize("realonly", [False, True])
def test_operator_symmetries(realonly):
    from dirac_caspt2_gb300 import synth
    S = synth.make_system(synth.SynthConfig(4, 4, 8, 2, seed=2, realonly=realonly))
    h, n = S.h, S.nmo
    p = np.arange(n) ^ 1
    assert np.abs(h - h.conj().T).max() == 0.0
    assert np.abs(h[np.ix_(p, p)] - _tr_sign(n) * h.conj()).max() == 0.0
    # Kramers pairs have bit-identical orbital energies, distinct pairs differ
    assert np.all(S.mo_energy[0::2] == S.mo_energy[1::2])
    assert len(np.unique(S.mo_energy)) == n // 2
    g = S.dense_g()
    assert np.abs(g - g.transpose(2, 3, 0, 1)).max() < 1e-15                 # (pq|rs) = (rs|pq)
    assert np.abs(g - g.transpose(1, 0, 3, 2).conj()).max() < 1e-15          # (pq|rs) = (qp|sr)*
    s = _tr_sign(n)
    # (q~ p~|rs) = (-1)^(p+q) (pq|rs)   (module_2integrals.F90:395-434)
    assert np.abs(g[np.ix_(p, p, np.arange(n), np.arange(n))].transpose(1, 0, 2, 3)
                  - s[:, :, None, None] * g).max() < 1e-15


def test_canonical_records_reproduce_dense_tensor():
    from dirac_caspt2_gb300 import synth
    from oracle import caspt2_oracle as O
    S = synth.make_system(synth.SynthConfig(4, 4, 8, 2, seed=1))
    g = S.dense_g()
    sysm = O.System(ninact=4, nact=4, nsec=8, nelec=2, nmo=S.nmo, nsymrpa=1, multb=S.multb, irpamo=S.irpamo,
                    h=S.h, ecore=S.ecore, rec_idx=S.rec_idx, rec_val=S.rec_val, realonly=False)
    ints = O.Integrals(sysm)
    rng = {1: (0, 4), 2: (4, 8), 3: (8, 16)}
    read = list(O.Integrals.PATTERNS) + [p for p in itertools.product((1, 2), repeat=4)]
    for sp in read:
        assert synth._used_pattern(sp)
        r = [rng[x] for x in sp]
        ref = g[r[0][0]:r[0][1], r[1][0]:r[1][1], r[2][0]:r[2][1], r[3][0]:r[3][1]]
        assert np.abs(ints.block(sp) - ref).max() < 1e-16, sp


def test_generator_is_deterministic():
    from dirac_caspt2_gb300 import synth
    a = synth.make_system(synth.SynthConfig(4, 2, 6, 1, seed=9))
    b = synth.make_system(synth.SynthConfig(4, 2, 6, 1, seed=9))
    assert np.array_equal(a.rec_idx, b.rec_idx) and np.array_equal(a.rec_val, b.rec_val)
    assert np.array_equal(a.h, b.h)

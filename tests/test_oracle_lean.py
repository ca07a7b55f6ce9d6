"""The oracle's lean mode (inputs released once read, for the largest fixtures) gives the same
numbers as the default mode."""
import numpy as np


def test_lean_mode_same_numbers():
    from dirac_caspt2_gb300 import synth
    from oracle import caspt2_oracle as O
    S = synth.make_system(synth.SynthConfig(4, 6, 12, 3, seed=8))
    mk = lambda: O.System(ninact=4, nact=6, nsec=12, nelec=3, nmo=S.nmo, nsymrpa=1, multb=S.multb,
                          irpamo=S.irpamo, h=S.h, ecore=S.ecore, rec_idx=S.rec_idx.copy(),
                          rec_val=S.rec_val.copy(), realonly=False)
    a = O.run(mk())
    s = mk()
    b = O.run(s, lean=True)
    assert len(s.rec_val) == 0
    assert a.total_energy == b.total_energy
    for k in a.e2:
        assert a.e2[k] == b.e2[k] and a.sumc2[k] == b.sumc2[k]

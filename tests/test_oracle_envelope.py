"""The reference's E-subspace energy is the only quantity that depends on the eigenvector
choice inside degenerate active Kramers pairs (complex systems without point-group
symmetry); all other subspaces are invariant.  For real systems E is invariant too."""
import numpy as np


def _sys(realonly):
    from dirac_caspt2_gb300 import synth
    from oracle import caspt2_oracle as O
    S = synth.make_system(synth.SynthConfig(4, 4, 8, 2, seed=1, realonly=realonly))
    return O.System(ninact=4, nact=4, nsec=8, nelec=2, nmo=S.nmo, nsymrpa=1, multb=S.multb, irpamo=S.irpamo,
                    h=S.h, ecore=S.ecore, rec_idx=S.rec_idx, rec_val=S.rec_val, realonly=realonly)


def test_only_E_depends_on_active_pair_rotation():
    from oracle import caspt2_oracle as O
    s = _sys(False)
    base = O.run(s)
    rot = O.run(s, active_pair_rotation=np.random.default_rng(1))
    for k in "ABCDFGH":
        assert abs(rot.e2[k] - base.e2[k]) < 1e-15
    lo, hi = O.e_subspace_envelope(s, trials=4)
    assert lo <= base.e2["E"] <= hi
    assert hi - lo < 1e-8


def test_real_systems_are_rotation_invariant():
    from oracle import caspt2_oracle as O
    s = _sys(True)
    lo, hi = O.e_subspace_envelope(s, trials=3)
    assert hi - lo < 1e-15

"""Independent eigensolver chains (divide and conquer, back-transformations, tridiagonal-form
E2) forked onto a context's auxiliary streams: the same arithmetic as on one stream, so the
energies agree to the bit with DCG_EIG_STREAMS=1."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_forked_eigensolver_chains_match_one_stream(gpu_lib, monkeypatch, prec):
    from dirac_caspt2_gb300 import api, synth
    p = api.DCG_PREC_SPLIT if prec == "split" else api.DCG_PREC_FP64
    s = api.SystemInput.from_synth(synth.make_system(synth.SynthConfig(12, 8, 120, 4, seed=5)))
    prev = api.autotune_mode(0)   # the same GEMM choices in both contexts
    try:
        monkeypatch.setenv("DCG_EIG_STREAMS", "1")
        with api.Caspt2Session(0, p) as ses:
            one = ses.solve(s)
        monkeypatch.setenv("DCG_EIG_STREAMS", "4")
        with api.Caspt2Session(0, p) as ses:
            four = ses.solve(s)
            again = ses.solve(s)
    finally:
        api.autotune_mode(prev)
    assert four.total_energy == one.total_energy
    assert again.total_energy == one.total_energy
    for k in one.e2:
        assert four.e2[k] == one.e2[k]

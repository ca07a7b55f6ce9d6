"""The Cholesky route of the A and C Gram blocks (dcg_set_metric_solver AUTO: when the
metric K = G G^H has no eigenvalue under the 1e-8 cutoff, E2 = -u^H (D + alpha)^-1 u with
u = K^-1 G v; with a few under it, the same on the complement of their eigenvectors) against
the eigendecomposition route (EIGEN) on the same systems, complex and real, FP64 and split:
every subspace's e2 and sumc2 within 1e-10 Eh (stated tolerance), and the oracle within
1e-9 Eh."""
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _run(s, metric, prec):
    from dirac_caspt2_gb300 import api
    with api.Caspt2Session(0, prec) as ses:
        ses.set_metric_solver(metric)
        r = ses.solve(s)
        return r, ses.gram_cholesky_blocks()


# deflated: the metric has eigenvalues under the cutoff (5 at 10 active spinors), which the
# route projects out instead of falling back to the eigendecompositions
@pytest.mark.parametrize("dims,realonly,deflated", [((4, 8, 20, 4), False, False), ((6, 6, 24, 3), False, False),
                                                    ((4, 8, 16, 4), True, False), ((2, 10, 12, 5), False, True)])
@pytest.mark.parametrize("prec", [0, 1])
def test_cholesky_route_matches_eigen_route(gpu_lib, dims, realonly, deflated, prec):
    from dirac_caspt2_gb300 import api, synth
    S = synth.make_system(synth.SynthConfig(*dims, seed=31, realonly=realonly))
    s = api.SystemInput.from_synth(S)
    with api.Caspt2Session(0, prec) as ses:
        ses.set_metric_solver("auto")
        a = ses.solve(s)
        na, nd = ses.gram_cholesky_blocks(), ses.gram_deflated_blocks()
        ses.set_metric_solver("eigen")
        e = ses.solve(s)
        ne = ses.gram_cholesky_blocks()
    assert na > 0 and ne == 0
    assert (nd > 0) == deflated
    for k in "ABCDEFGH":
        assert abs(a.e2[k] - e.e2[k]) <= TOL, (k, a.e2[k], e.e2[k])
        assert abs(a.sumc2[k] - e.sumc2[k]) <= TOL, k
    assert abs(a.total_energy - e.total_energy) <= TOL


def test_cholesky_route_matches_oracle(gpu_lib):
    from dirac_caspt2_gb300 import api, synth
    from oracle import caspt2_oracle as O
    from conftest import oracle_system
    S = synth.make_system(synth.SynthConfig(4, 8, 20, 4, seed=32))
    s = api.SystemInput.from_synth(S)
    r, n = _run(s, "auto", 0)
    ref = O.run(oracle_system(s))
    assert n > 0
    for k in "AC":
        assert abs(r.e2[k] - ref.e2[k]) <= 1e-9, k
        assert abs(r.sumc2[k] - ref.sumc2[k]) <= 1e-9, k
    assert abs(r.total_energy - ref.total_energy) <= 1e-8

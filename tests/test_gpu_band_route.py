"""E2 of the B' blocks from a band form (stage one of a two-stage Hermitian reduction, then one
banded solve with partial pivoting per outer index) against the tridiagonal-form route and the
oracle.  DCG_BPRIME_ROUTE=band forces the band route on every B' block that would take the
tridiagonal form (the Gram blocks of A and C and the S/B-route blocks of B, D-G), on systems
small enough for the oracle (even electron counts: a nondegenerate CASCI root).  The band route
is not the default (it measured slower than the tridiagonal form on GB300).
Tolerances: every subspace within 1e-9 Eh of the oracle, the two routes within 1e-11 Eh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from conftest import oracle_system

SYS = [(4, 8, 12, 4, 0, False), (6, 8, 20, 4, 1, False), (4, 10, 8, 4, 2, True)]


@pytest.mark.parametrize("ni,na,ns,ne,seed,realonly", SYS)
def test_band_route_matches_tridiagonal_route_and_oracle(gpu_lib, monkeypatch, ni, na, ns, ne, seed, realonly):
    from dirac_caspt2_gb300 import api, synth
    from oracle import caspt2_oracle as O
    S = synth.make_system(synth.SynthConfig(ni, na, ns, ne, seed=seed, realonly=realonly))
    s = api.SystemInput.from_synth(S)
    out = {}
    for route in ("tridiag", "band"):
        monkeypatch.setenv("DCG_BPRIME_ROUTE", route)
        with api.Caspt2Session(0) as ses:
            ses.set_metric_solver("eigen")   # the Gram blocks through B' (not the Cholesky route)
            out[route] = ses.solve(s)
    ref = O.run(oracle_system(s))
    for k in "ABCDEFGH":
        assert abs(out["band"].e2[k] - out["tridiag"].e2[k]) <= 1e-11, k
        assert abs(out["band"].sumc2[k] - out["tridiag"].sumc2[k]) <= 1e-11, k
        assert abs(out["band"].e2[k] - ref.e2[k]) <= 1e-9, k
    assert abs(out["band"].total_energy - ref.total_energy) <= 1e-9

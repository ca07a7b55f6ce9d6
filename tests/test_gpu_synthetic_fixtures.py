"""The benchmark systems at their full sizes against committed oracle energies: the seeded
synthetic 8/6/40 (4 electrons) and 20/12/300 (6 electrons) systems, and 40/14/160 (8 electrons:
the active space and inactive count of the 40/14/800 large solve, 3003 determinants, with the
secondary space cut to what the CPU oracle finishes in minutes), whose CPU-oracle results
tests/golden/make_synthetic_fixtures.py stored in tests/golden/synthetic_<name>.json.  Both GPU
paths, FP64 and split precision, are held to the stated targets: CASCI and every subspace's
e2X within 1e-9 Eh, the total within 1e-8 Eh (sumc2,X within 1e-9)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from conftest import GOLDEN_DIR

TOL_SUB = 1e-9
TOL_TOTAL = 1e-8


@pytest.fixture(scope="module", params=["cas_8_6_40", "cas_20_12_300", "cas_40_14_160"])
def case(request):
    from dirac_caspt2_gb300 import api, synth
    ref = json.load(open(os.path.join(GOLDEN_DIR, f"synthetic_{request.param}.json")))
    S = synth.make_system(synth.CONFIGS[request.param])
    v = np.asarray(S.rec_val)
    fp = ref["fingerprint"]
    assert len(v) == fp["nrec"] and S.nmo == fp["nmo"]
    assert float(np.sum(v.real)) == pytest.approx(fp["sum_re"], rel=1e-9, abs=1e-9)
    assert float(np.sum(np.abs(v))) == pytest.approx(fp["sum_abs"], rel=1e-9)
    assert float(np.sum(S.h.real)) == pytest.approx(fp["sum_h_re"], rel=1e-9)
    return api.SystemInput.from_synth(S), ref


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_benchmark_system_matches_oracle_fixture(gpu_lib, case, precision):
    from dirac_caspt2_gb300 import api
    s, ref = case
    prec = api.DCG_PREC_SPLIT if precision == "split" else api.DCG_PREC_FP64
    with api.Caspt2Session(0, prec) as ses:
        r = ses.solve(s)
    assert r.ndet == ref["ndet"]
    assert abs(r.casci_energies[0] - ref["casci"]) <= TOL_SUB
    for k in "ABCDEFGH":
        assert abs(r.e2[k] - ref["e2"][k]) <= TOL_SUB, (k, r.e2[k], ref["e2"][k])
        assert abs(r.sumc2[k] - ref["sumc2"][k]) <= TOL_SUB, (k, r.sumc2[k], ref["sumc2"][k])
    assert abs(r.total_energy - ref["total"]) <= TOL_TOTAL

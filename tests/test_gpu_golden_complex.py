"""The reference's four runnable golden cases through the library's own readers and the full
GPU path, with MDCINT in the real-only layout and rewritten in the complex layout (zero
imaginary parts, so the reader reports a complex system as module_realonly.F90:29-77 decides).
The complex layout takes the complex reader, the complex canonicalisation and the complex
record scatter; both layouts, on the FP64 and the split-precision path, reproduce every printed
energy of reference.<case>.out within 1e-10 Eh: CASCI, e2X and sumc2,X of every subspace, the
per-irrep e2X(isym) lines (solve_A_subspace.F90:262 and its B..G counterparts, the same set of
lines) and the total."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from conftest import GOLDEN_CASES, GOLDEN_DIR
from test_mdcint import write_case_dir
from test_oracle_golden import check_e2_sym

TOL = 1e-10


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("layout", ["complex", "real"])
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_through_native_readers(gpu_lib, tmp_path, case, layout, precision):
    from dirac_caspt2_gb300 import api
    inp = write_case_dir(case, str(tmp_path), complex_layout=(layout == "complex"))
    prec = api.DCG_PREC_SPLIT if precision == "split" else api.DCG_PREC_FP64
    with api.NativeFiles(str(tmp_path), inp) as nf:
        assert nf.realonly == (layout == "real")
        s = nf.system_input()
        with api.Caspt2Session(0, prec) as ses:
            ses.set_system_mdcint(s, nf)
            eig, _ = ses.casci(max(1, s.selectroot))
            e2, sc2, e0, et = ses.caspt2()
            e2_sym = ses.caspt2_irreps()[0]
    g = np.load(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    assert abs(eig[s.selectroot - 1] - float(g["ref_casci"])) < TOL
    for i, k in enumerate("ABCDEFGH"):
        ref = g["ref_e2"][i]
        if np.isnan(ref):   # skipped by the reference (ninact = 0 or nsec = 0)
            assert e2[k] == 0.0 and sc2[k] == 0.0
            continue
        assert abs(e2[k] - ref) < TOL, (k, e2[k], ref)
        assert abs(sc2[k] - g["ref_sumc2"][i]) < TOL, (k, sc2[k], g["ref_sumc2"][i])
    check_e2_sym(e2_sym, g["ref_e2_sym"])
    assert abs(et - float(g["ref_total"])) < TOL

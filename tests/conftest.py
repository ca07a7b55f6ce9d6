import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["c2_h2o_dev", "check_minelecras3_dev", "ninact_0_h2_dev", "mdcint_scheme_6_dirac23_c32h_n2_dev"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


def oracle_system(s):
    """oracle.System from an api.SystemInput."""
    from oracle import caspt2_oracle as O
    return O.System(ninact=s.ninact, nact=s.nact, nsec=s.nsec, nelec=s.nelec, nmo=s.nmo, nsymrpa=s.nsymrpa,
                    multb=np.asarray(s.multb), irpamo=np.asarray(s.irpamo), h=np.asarray(s.h), ecore=s.ecore,
                    rec_idx=np.asarray(s.rec_idx), rec_val=np.asarray(s.rec_val), realonly=s.realonly,
                    totsym=s.totsym, selectroot=s.selectroot, eshift=s.eshift,
                    ras1=tuple(range(s.ras[0])), ras2=tuple(range(s.ras[1])), ras3=tuple(range(s.ras[2])),
                    ras1_max_hole=s.ras1_max_hole, ras3_max_elec=s.ras3_max_elec,
                    min_hole_ras1=s.min_hole_ras1, min_elec_ras3=s.min_elec_ras3)


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load the CUDA library; fail loudly without it."""
    from dirac_caspt2_gb300 import build, api
    build.build()
    return api.load_library()

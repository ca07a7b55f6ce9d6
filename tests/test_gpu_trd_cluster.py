"""The cluster form of the Householder tridiagonalisation (one thread-block cluster per
matrix of order <= 400, exchanging through distributed shared memory; an option, selected by
DCG_TRD_CLUSTER=1, read once per process) against the default cooperative grid-wide form:
both use the same arithmetic and summation orders, so dcg_heev gives the same bits either
way.  The cluster form runs in a child process.  The orders cover every cluster shape: 1, 4
and 16 blocks."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORDERS = (1, 2, 7, 40, 90, 150, 250, 300, 400)


def _matrix(n):
    rng = np.random.default_rng(1000 + n)
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return a + a.conj().T


CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, {root!r})
from dirac_caspt2_gb300 import api
from tests.test_gpu_trd_cluster import ORDERS, _matrix
out = {{}}
with api.Caspt2Session(0) as s:
    for n in ORDERS:
        w, z = s.heev(_matrix(n))
        out[str(n)] = [w.tobytes().hex(), z.tobytes().hex()]
print(json.dumps(out))
"""


def test_cluster_form_matches_cooperative_form_bit_for_bit(gpu_lib, tmp_path):
    from dirac_caspt2_gb300 import api
    env = dict(os.environ, DCG_TRD_CLUSTER="1")
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    clus = json.loads(r.stdout.strip().splitlines()[-1])
    with api.Caspt2Session(0) as s:
        for n in ORDERS:
            a = _matrix(n)
            w, z = s.heev(a)
            wr = np.linalg.eigvalsh(a)
            scale = max(1.0, np.abs(wr).max())
            assert np.abs(w - wr).max() <= 1e-12 * scale, n
            assert np.abs(a @ z - z * w).max() <= 1e-12 * scale, n
            assert w.tobytes().hex() == clus[str(n)][0], f"eigenvalues differ at n={n}"
            assert z.tobytes().hex() == clus[str(n)][1], f"eigenvectors differ at n={n}"

"""Merged Householder reductions (dcg_set_merge_reductions): two contexts that reduce their
matrices at the same time share one cooperative launch, and each matrix gets the same bits as
when it is reduced alone.  A merge window (DCG_MERGE_WINDOW_US) makes the two submissions meet
deterministically: the first waits for the second before the launch."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _herm(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return X + X.conj().T


@pytest.mark.parametrize("n0,n1", [(300, 300), (792, 180), (520, 520)])
def test_two_contexts_share_one_launch(gpu_lib, monkeypatch, n0, n1):
    from dirac_caspt2_gb300 import api
    mats = [_herm(n0, 1), _herm(n1, 2)]
    alone = []
    for H in mats:
        with api.Caspt2Session(0) as ses:
            alone.append(ses.heev(H))
    monkeypatch.setenv("DCG_MERGE_WINDOW_US", "2000000")
    sessions = [api.Caspt2Session(0), api.Caspt2Session(0)]
    for ses in sessions:
        assert ses.lib.dcg_set_merge_reductions(ses.h, 1) == 0
    out = [None, None]
    err = []

    def run(q):
        try:
            out[q] = sessions[q].heev(mats[q])
        except Exception as e:   # reported below
            err.append(e)

    m0 = api.merged_reduction_stats(0)
    th = [threading.Thread(target=run, args=(q,)) for q in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join(60)
    for ses in sessions:
        ses.close()
    assert not err, err
    m1 = api.merged_reduction_stats(0)
    assert m1["joint_launches"] - m0["joint_launches"] >= 1
    assert m1["submissions"] - m0["submissions"] >= 2
    for q in range(2):
        w, Z = out[q]
        w0, Z0 = alone[q]
        assert np.array_equal(w, w0)
        assert np.array_equal(Z, Z0)

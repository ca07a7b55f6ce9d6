"""Bounded device-side waits that run out, on the GPU, without a fault: with a wait limit of
1 ns (dcg_set_wait_limit) the pipeline waits of the tensor-core split GEMM (both kernels, the
one-tile and the persistent one) and the grid-barrier and published-reflector waits of the
Householder tridiagonalisation give up.  The kernel then leaves cleanly (copies in flight land
and issued tensor-core operations complete before a CTA frees its tensor memory), the call
returns DCG_E_NUMERIC with the reason, and the same context, with the default limits
restored, gives the same results as before, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", ["0", "2"])   # one-tile kernel, persistent kernel
def test_split_gemm_wait_runs_out_and_context_recovers(gpu_lib, monkeypatch, kernel):
    torch = pytest.importorskip("torch")
    from dirac_caspt2_gb300 import api
    monkeypatch.setenv("DCG_SPLIT_KERNEL", kernel)
    M, N, K = 2048, 128, 512
    rng = np.random.default_rng(3)
    A = rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))
    B = rng.normal(size=(K, N)) + 1j * rng.normal(size=(K, N))
    dev = lambda x: torch.from_numpy(np.asfortranarray(x).ravel(order="F").view(np.float64).copy()).cuda()
    dA, dB = dev(A), dev(B)
    dC = torch.zeros(2 * M * N, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    args = lambda: (api.DCG_PREC_SPLIT, M, N, K, 1, dA.data_ptr(), 1, M, 0, dB.data_ptr(), K, False,
                    dC.data_ptr(), 1, M, 0)
    with api.Caspt2Session(0, api.DCG_PREC_SPLIT) as ses:
        ses.zgemm(*args())
        ref = dC.cpu().numpy().copy()
        C = ref.view(np.complex128).reshape(N, M).T
        assert np.abs(C - A @ B).max() <= 1e-9 * np.abs(A).max() * np.abs(B).max() * K
        ses.set_wait_limit(1e-9)
        with pytest.raises(api.DcgError) as ei:
            ses.zgemm(*args())
        assert ei.value.code == -6 and "timed out" in str(ei.value)
        ses.set_wait_limit(0)
        dC.zero_()
        ses.zgemm(*args())
        assert np.array_equal(dC.cpu().numpy(), ref)


def test_tridiagonalisation_wait_runs_out_and_context_recovers(gpu_lib):
    from dirac_caspt2_gb300 import api
    n = 600
    rng = np.random.default_rng(4)
    X = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    H = X + X.conj().T
    with api.Caspt2Session(0) as ses:
        w_ref = ses.heev(H, vectors=False)
        assert np.abs(w_ref - np.linalg.eigvalsh(H)).max() <= 1e-10 * np.abs(w_ref).max()
        ses.set_wait_limit(1e-9)
        raised = 0
        for _ in range(3):   # a wait gives up once a block has polled for longer than the limit
            try:
                w = ses.heev(H, vectors=False)
                assert np.array_equal(w, w_ref)   # no wait ran out: the result is unchanged
            except api.DcgError as e:
                assert e.code == -6 and "timed out" in str(e)
                raised += 1
        assert raised > 0
        ses.set_wait_limit(0)
        assert np.array_equal(ses.heev(H, vectors=False), w_ref)

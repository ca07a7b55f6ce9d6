"""The split-precision tensor-core complex GEMM (dcg_zgemm, DCG_PREC_SPLIT) against a
complex128 reference (torch.matmul in FP64 on the device).

Error bound per element: each operand is cut at 2^-36 of its row / column maximum, so
|C - C_ref|(i, j) <= 4e-11 * K * max_k |A(i, k)| * max_k |B(k, j)| (2^-36 ~ 1.5e-11, with
margin for the summation)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SPLIT = 1


def _rand(shape, gen):
    return (torch.randn(shape, dtype=torch.float64, generator=gen) +
            1j * torch.randn(shape, dtype=torch.float64, generator=gen)).to(torch.complex128)


@pytest.fixture(scope="module")
def session(gpu_lib):
    from dirac_caspt2_gb300 import api
    s = api.Caspt2Session(0)
    yield s
    s.close()


def _check(C, Cref, A_rowmax, B_colmax, K):
    bound = 4e-11 * K * (A_rowmax[:, None] * B_colmax[None, :]) + 1e-300
    err = (C - Cref).abs()
    ratio = (err / bound).max().item()
    assert ratio <= 1.0, f"split GEMM error {ratio:.3g} x bound"


@pytest.mark.parametrize("M,N,K,batch,conj", [(128, 64, 8, 1, False), (300, 40, 50, 1, False),
                                              (130, 20, 33, 3, True), (1000, 300, 300, 2, True),
                                              (257, 7, 600, 1, False), (64, 129, 129, 1, True)])
def test_split_gemm_column_major(session, M, N, K, batch, conj):
    gen = torch.Generator().manual_seed(M + 7 * N + 13 * K + batch)
    A = _rand((batch, K, M), gen).transpose(1, 2)          # column-major M x K per batch
    # spread row magnitudes over 12 decades
    A = A * torch.logspace(-6, 6, M, dtype=torch.float64)[None, :, None]
    B = _rand((N, K), gen).T                               # column-major K x N
    A_cm = torch.empty((batch, K, M), dtype=torch.complex128, device="cuda")
    A_cm.copy_(A.transpose(1, 2))
    B_cm = torch.empty((N, K), dtype=torch.complex128, device="cuda")
    B_cm.copy_(B.T)
    C = torch.zeros((batch, N, M), dtype=torch.complex128, device="cuda")
    session.zgemm(SPLIT, M, N, K, batch, A_cm.data_ptr(), 1, M, M * K, B_cm.data_ptr(), K, conj,
                  C.data_ptr(), 1, M, M * N)
    torch.cuda.synchronize()
    Bop = B.conj() if conj else B
    Cref = torch.matmul(A.cuda(), Bop.cuda())              # (batch, M, N)
    Cgot = C.transpose(1, 2)
    _check(Cgot, Cref, A.abs().amax(dim=(0, 2)).cuda(), B.abs().amax(dim=0).cuda(), K)


def test_split_gemm_k_contiguous_and_transposed_output(session):
    """The left-multiply form of the transformation: C = U^H T computed as C^T = T^T conj(U),
    with T^T rows contiguous along K and C written transposed."""
    gen = torch.Generator().manual_seed(5)
    K, Nbig, Msmall = 70, 900, 70
    T = _rand((Nbig, K), gen)                              # T column-major K x Nbig == row-major Nbig x K
    U = _rand((K, Msmall), gen)
    T_d = T.cuda().contiguous()                            # element (n, k) at n*K + k
    U_cm = torch.empty((Msmall, K), dtype=torch.complex128, device="cuda")
    U_cm.copy_(U.T)                                        # column-major K x Msmall
    C = torch.zeros((Nbig, Msmall), dtype=torch.complex128, device="cuda")   # C^T row-major = C col-major
    session.zgemm(SPLIT, Nbig, Msmall, K, 1, T_d.data_ptr(), K, 1, 0, U_cm.data_ptr(), K, True,
                  C.data_ptr(), Msmall, 1, 0)
    torch.cuda.synchronize()
    Cref = torch.matmul(T.cuda(), U.conj().cuda())
    _check(C, Cref, T.abs().amax(dim=1).cuda(), U.abs().amax(dim=0).cuda(), K)


def test_split_gemm_zero_rows_and_columns(session):
    gen = torch.Generator().manual_seed(9)
    M, N, K = 200, 30, 40
    A = _rand((M, K), gen)
    A[5] = 0
    A[199] = 0
    B = _rand((K, N), gen)
    B[:, 3] = 0
    A_cm = A.T.contiguous().cuda()
    B_cm = B.T.contiguous().cuda()
    C = torch.full((N, M), 7.0 + 0j, dtype=torch.complex128, device="cuda")
    session.zgemm(SPLIT, M, N, K, 1, A_cm.data_ptr(), 1, M, 0, B_cm.data_ptr(), K, False, C.data_ptr(), 1, M, 0)
    torch.cuda.synchronize()
    Cref = (A @ B).cuda()
    assert torch.all(C.T[5] == 0) and torch.all(C.T[199] == 0) and torch.all(C.T[:, 3] == 0)
    _check(C.T, Cref, A.abs().amax(dim=1).cuda(), B.abs().amax(dim=0).cuda(), K)


def test_split_gemm_accumulate(session):
    gen = torch.Generator().manual_seed(11)
    M, N, K = 150, 25, 30
    A = _rand((M, K), gen)
    B = _rand((K, N), gen)
    C0 = _rand((M, N), gen)
    A_cm = A.T.contiguous().cuda()
    B_cm = B.T.contiguous().cuda()
    C = C0.T.contiguous().cuda()
    session.zgemm(SPLIT, M, N, K, 1, A_cm.data_ptr(), 1, M, 0, B_cm.data_ptr(), K, False, C.data_ptr(), 1, M, 0,
                  accumulate=True)
    torch.cuda.synchronize()
    Cref = (C0 + A @ B).cuda()
    _check(C.T, Cref, A.abs().amax(dim=1).cuda(), B.abs().amax(dim=0).cuda(), K)


@pytest.mark.parametrize("M,N,K,batch", [(1000, 300, 300, 2), (257, 7, 600, 1), (130, 33, 40, 3), (64, 129, 129, 1)])
def test_split_gemm_kernel_variants_agree(session, monkeypatch, M, N, K, batch):
    """The four tuned variants (row- or column-block raster, one tile per CTA or persistent
    CTAs with double-buffered accumulators) give the same bits, and those pass the bound."""
    gen = torch.Generator().manual_seed(3 * M + N + K)
    A = _rand((batch, K, M), gen).transpose(1, 2)
    B = _rand((N, K), gen).T
    A_cm = torch.empty((batch, K, M), dtype=torch.complex128, device="cuda")
    A_cm.copy_(A.transpose(1, 2))
    B_cm = torch.empty((N, K), dtype=torch.complex128, device="cuda")
    B_cm.copy_(B.T)
    out = []
    for q in "0123":
        monkeypatch.setenv("DCG_SPLIT_KERNEL", q)
        C = torch.zeros((batch, N, M), dtype=torch.complex128, device="cuda")
        session.zgemm(SPLIT, M, N, K, batch, A_cm.data_ptr(), 1, M, M * K, B_cm.data_ptr(), K, False,
                      C.data_ptr(), 1, M, M * N)
        torch.cuda.synchronize()
        out.append(C.clone())
    for C in out[1:]:
        assert torch.equal(C, out[0])
    Cref = torch.matmul(A.cuda(), B.cuda())
    _check(out[2].transpose(1, 2), Cref, A.abs().amax(dim=(0, 2)).cuda(), B.abs().amax(dim=0).cuda(), K)


@pytest.mark.parametrize("M,N,K,batch,conj", [(128, 64, 8, 1, False), (300, 40, 50, 1, False),
                                              (130, 20, 33, 3, True), (792, 300, 1728, 1, False),
                                              (64, 129, 129, 1, True)])
def test_split_gemm_seven_slices(session, M, N, K, batch, conj):
    """The seven-slice product (DCG_PREC_SPLIT_ACC): within 1e-13 * K * row max * column max
    (2^-45 ~ 2.8e-14 per term), and far more accurate than the five-slice product on the same
    operands (the Gram metric and the products Lambda^-1 amplifies take it)."""
    from dirac_caspt2_gb300 import api
    gen = torch.Generator().manual_seed(M + 5 * N + 11 * K + batch)
    A = _rand((batch, K, M), gen).transpose(1, 2)
    A = A * torch.logspace(-6, 6, M, dtype=torch.float64)[None, :, None]
    B = _rand((N, K), gen).T
    A_cm = torch.empty((batch, K, M), dtype=torch.complex128, device="cuda")
    A_cm.copy_(A.transpose(1, 2))
    B_cm = torch.empty((N, K), dtype=torch.complex128, device="cuda")
    B_cm.copy_(B.T)
    out = {}
    for prec in (SPLIT, api.DCG_PREC_SPLIT_ACC):
        C = torch.zeros((batch, N, M), dtype=torch.complex128, device="cuda")
        session.zgemm(prec, M, N, K, batch, A_cm.data_ptr(), 1, M, M * K, B_cm.data_ptr(), K, conj,
                      C.data_ptr(), 1, M, M * N)
        torch.cuda.synchronize()
        out[prec] = C.transpose(1, 2)
    Bop = B.conj() if conj else B
    Cref = torch.matmul(A.cuda(), Bop.cuda())
    rmax, cmax = A.abs().amax(dim=(0, 2)).cuda(), B.abs().amax(dim=0).cuda()
    scale = K * (rmax[:, None] * cmax[None, :])
    acc = ((out[api.DCG_PREC_SPLIT_ACC] - Cref).abs() / scale).max().item()
    five = ((out[SPLIT] - Cref).abs() / scale).max().item()
    assert acc <= 1e-13, acc
    assert acc * 50 <= five or five <= 1e-13, (acc, five)

"""The device Hermitian eigensolver (dcg_heev: Householder tridiagonalisation, divide and
conquer, back-transformation) against LAPACK through numpy, on the spectra the CASPT2 path
produces: Kramers-degenerate Hermitian matrices, rank-deficient overlap-like (Gram)
matrices, exact multiplicities, tight clusters, and trivial cases.

Bounds (relative to max |eigenvalue|): eigenvalues within 1e-12, residual
max |A z - w z| within 1e-12, orthogonality max |Z^H Z - I| within 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _kramers(rng, h):
    a = rng.normal(size=(h, h)) + 1j * rng.normal(size=(h, h))
    a = a + a.conj().T
    b = rng.normal(size=(h, h)) + 1j * rng.normal(size=(h, h))
    b = b - b.T
    return np.block([[a, b], [-b.conj(), a.conj()]])


def _gram(rng, rank, n, cplx=True):
    g = rng.normal(size=(rank, n)) + (1j * rng.normal(size=(rank, n)) if cplx else 0)
    return g.conj().T @ g / n


def _cases():
    rng = np.random.default_rng(2024)
    out = {}
    for n in (1, 2, 3, 17, 64, 100, 257):
        a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        out[f"random_{n}"] = a + a.conj().T
    out["real_symmetric_300"] = (lambda x: x + x.T)(rng.normal(size=(300, 300)))
    out["kramers_200"] = _kramers(rng, 100)
    out["kramers_498"] = _kramers(rng, 249)
    out["gram_rank120_400"] = _gram(rng, 120, 400)
    out["gram_rank496_1000"] = _gram(rng, 496, 1000)
    # the A/C metric order at 12 active spinors and the largest shared-memory order
    out["gram_rank700_792"] = _gram(rng, 700, 792)
    out["random_1400"] = (lambda x: x + x.conj().T)(rng.normal(size=(1400, 1400)) + 1j * rng.normal(size=(1400, 1400)))
    out["gram_real_rank50_333"] = _gram(rng, 50, 333, cplx=False)
    q, _ = np.linalg.qr(rng.normal(size=(150, 150)) + 1j * rng.normal(size=(150, 150)))
    w = np.repeat([-1.0, 0.0, 2.0, 5.0, 5.0 + 1e-13], 30)
    out["multiplicity_150"] = (q * w) @ q.conj().T
    out["tight_cluster_120"] = (q[:120, :120] * 0 + np.eye(120)) + 1e-11 * (lambda x: x + x.conj().T)(
        rng.normal(size=(120, 120)) + 1j * rng.normal(size=(120, 120)))
    out["zero_50"] = np.zeros((50, 50), complex)
    out["identity_50"] = np.eye(50, dtype=complex)
    out["diagonal_80"] = np.diag(rng.normal(size=80)).astype(complex)
    return out


CASES = _cases()


@pytest.fixture(scope="module")
def session(gpu_lib):
    from dirac_caspt2_gb300 import api
    s = api.Caspt2Session(0)
    yield s
    s.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_heev_matches_lapack(session, name):
    a = CASES[name]
    n = a.shape[0]
    w, z = session.heev(a)
    wr = np.linalg.eigvalsh(a)
    scale = max(1.0, np.abs(wr).max())
    assert np.all(np.diff(w) >= 0), "eigenvalues not ascending"
    assert np.abs(w - wr).max() <= TOL * scale
    assert np.abs(a @ z - z * w).max() <= TOL * scale
    assert np.abs(z.conj().T @ z - np.eye(n)).max() <= TOL


def test_heev_deterministic(session):
    a = CASES["kramers_200"]
    w1, z1 = session.heev(a)
    w2, z2 = session.heev(a)
    assert np.array_equal(w1, w2) and np.array_equal(z1, z2)


def test_heev_values_only(session):
    a = CASES["gram_rank120_400"]
    w = session.heev(a, vectors=False)
    assert np.abs(w - np.linalg.eigvalsh(a)).max() <= TOL * np.abs(w).max()


@pytest.mark.parametrize("n", [1, 2, 5, 64, 100, 333, 512, 1000, 7])
def test_stedc_matches_lapack(session, n):
    """The divide-and-conquer stage alone, on random tridiagonals of varied size.  The calls
    run in sequence on one session, so each one reuses the workspace the previous one left."""
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(100 + n)
    d, e = rng.normal(size=n), rng.normal(size=max(n - 1, 0))
    w, q = session.stedc(d, e)
    wr = scipy_linalg.eigh_tridiagonal(d, e, eigvals_only=True) if n > 1 else d.copy()
    t = np.diag(d) + (np.diag(e, 1) + np.diag(e, -1) if n > 1 else 0)
    scale = max(1.0, np.abs(wr).max())
    assert np.abs(w - wr).max() <= TOL * scale
    assert np.abs(t @ q - q * w).max() <= TOL * scale
    assert np.abs(q.T @ q - np.eye(n)).max() <= TOL


@pytest.mark.parametrize("n,nvec", [(100, 3), (300, 5), (700, 1), (700, 10), (900, 70)])
def test_heev_range_few_vectors(session, n, nvec):
    """Eigenvectors of the top nvec eigenvalues only: the few-column back-transformation (a
    CASCI root) and the many-column one, on both sides of 512 rows."""
    rng = np.random.default_rng(n + nvec)
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    a = a + a.conj().T
    w, z = session.heev_range(a, n - nvec)
    wr = np.linalg.eigvalsh(a)
    scale = max(1.0, np.abs(wr).max())
    assert np.abs(w - wr).max() <= TOL * scale
    ws = w[n - nvec:]
    assert np.abs(a @ z - z * ws).max() <= TOL * scale
    assert np.abs(z.conj().T @ z - np.eye(nvec)).max() <= TOL


def test_heev_batch_mixed_sizes(session):
    """The batched eigensolver on matrices of mixed size reduced together (the S and B'
    matrices of several subspace blocks): each result against LAPACK."""
    rng = np.random.default_rng(77)
    mats = []
    for n in (792, 496, 144, 66, 12, 1):
        a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        mats.append(a + a.conj().T)
    mats.append(CASES["gram_rank120_400"])
    mats.append(CASES["kramers_200"])
    for a, (w, z) in zip(mats, session.heev_batch(mats)):
        n = a.shape[0]
        wr = np.linalg.eigvalsh(a)
        scale = max(1.0, np.abs(wr).max())
        assert np.abs(w - wr).max() <= TOL * scale
        assert np.abs(a @ z - z * w).max() <= TOL * scale
        assert np.abs(z.conj().T @ z - np.eye(n)).max() <= TOL

"""The batched SCF's occupied-subspace eigensolver (Householder tridiagonalisation,
FP32 bisection, inverse iteration) against numpy.linalg.eigh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(qb, A, k, tol=1e-10):
    w, Y = qb.api.eigh_lowest(A, k)
    wr, Vr = np.linalg.eigh(A)
    scale = max(1.0, np.abs(wr).max())
    assert np.abs(w - wr[:k]).max() < tol * scale
    assert np.abs(Y.T @ Y - np.eye(k)).max() < tol
    assert np.abs(A @ Y - Y * w).max() < tol * scale
    if k < len(A) and wr[k] - wr[k - 1] > 1e-6 * scale:
        D, Dr = Y @ Y.T, Vr[:, :k] @ Vr[:, :k].T
        assert np.abs(D - Dr).max() < tol


@pytest.mark.parametrize("n,k", [(1, 1), (2, 1), (2, 2), (3, 1), (5, 3), (17, 8), (64, 30), (116, 58), (256, 100)])
def test_random_symmetric(qb, n, k):
    rng = np.random.default_rng(n)
    B = rng.normal(size=(n, n))
    _check(qb, B + B.T, k)


def test_degenerate_and_h2_like(qb):
    rng = np.random.default_rng(3)
    n = 40
    Q = np.linalg.qr(rng.normal(size=(n, n)))[0]
    w = np.sort(rng.normal(size=n))
    w[1] = w[0]
    w[5] = w[4] = w[3]
    _check(qb, Q @ np.diag(w) @ Q.T, 10)
    # symmetric two-centre matrix with equal diagonals (minimal-basis H2 in an orthonormal basis)
    _check(qb, np.array([[-0.6, -0.4], [-0.4, -0.6]]), 1)
    _check(qb, np.array([[-0.6, 0.4], [0.4, -0.6]]), 1)
    _check(qb, np.diag([3.0, -1.0, 2.0, -5.0]), 2)
    # the orthonormal-basis core Hamiltonian of minimal-basis H2 at 2.74 bohr: the first
    # bisection midpoint equals the diagonal, so a Sturm pivot is exactly zero
    S = np.array([[1.0, 0.2747943], [0.2747943, 1.0]])
    Hc = np.array([[-0.82913813, -0.34876032], [-0.34876032, -0.82913813]])
    w, U = np.linalg.eigh(S)
    X = U @ np.diag(w ** -0.5) @ U.T
    _check(qb, X.T @ Hc @ X, 1)
    # many matrices with equal diagonals and integer entries (exact pivots)
    rng = np.random.default_rng(9)
    for n in (3, 4, 6, 9):
        B = rng.integers(-3, 4, size=(n, n)).astype(float)
        A = B + B.T
        np.fill_diagonal(A, 1.0)
        _check(qb, A, max(1, n // 2))
    # block-diagonal copies of one block: every eigenvalue threefold, clusters across the
    # occupied/virtual boundary handled by the subspace test only
    B = rng.normal(size=(7, 7))
    blk = B + B.T
    A = np.kron(np.eye(3), blk)
    _check(qb, A, 9)
    # near-degenerate pairs (split 1e-7, inside the Gram-Schmidt cluster tolerance) and a
    # large diagonal shift
    Q = np.linalg.qr(rng.normal(size=(24, 24)))[0]
    w = np.repeat(np.sort(rng.normal(size=12)), 2)
    w[1::2] += 1e-7
    _check(qb, Q @ np.diag(w) @ Q.T, 12, tol=1e-9)
    _check(qb, 1e4 * np.eye(30) + (lambda M: M + M.T)(rng.normal(size=(30, 30))), 12, tol=1e-10)


def test_gap_inside_fp32_bracket(qb):
    # The gap between the highest occupied (k-1) and the lowest unoccupied (k) eigenvalue
    # below the FP32 bisection's resolution (~2.4e-7 ||T||): the eigensolver refines those
    # eigenvalues in FP64 and the occupied density still matches numpy's FP64 eigh, to the
    # accuracy such a gap allows any FP64 solver (~eps ||A|| / gap).
    rng = np.random.default_rng(21)
    for n, k, gap in ((20, 7, 1e-8), (48, 20, 3e-8), (64, 31, 1e-9), (116, 40, 5e-8)):
        Q = np.linalg.qr(rng.normal(size=(n, n)))[0]
        w = np.sort(rng.uniform(-2.0, 2.0, size=n))
        w[k] = w[k - 1] + gap
        A = Q @ np.diag(w) @ Q.T
        A = 0.5 * (A + A.T)
        wq, Y = qb.api.eigh_lowest(A, k)
        wr, Vr = np.linalg.eigh(A)
        scale = np.abs(wr).max()
        assert wr[k] - wr[k - 1] < 2.4e-7 * scale
        assert np.abs(wq - wr[:k]).max() < 1e-10 * scale
        D, Dr = Y @ Y.T, Vr[:, :k] @ Vr[:, :k].T
        assert np.abs(D - Dr).max() < max(100 * 2.220446049250313e-16 * scale / gap, 1e-10), (n, k, gap)

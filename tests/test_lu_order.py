"""The operation order of the complex64 LU with tensor-core updates
(lu_blocked_tc in optimet_gb300/csrc/solve.cu), restated in numpy: blocks of
128 columns factored as tall panels of 32 whose interchanges and updates stay
inside the block, the block's interchanges applied outside it afterwards, its
U rows solved 32 at a time, and one rank-128 trailing update. The order must
give P A = L U with the pivots of the unblocked right-looking order (each
panel's pivot search sees fully updated columns), which is what lets the GPU
tests compare the two paths. No GPU: the kernels themselves are checked by
tests/test_tensor_cores.py."""
import numpy as np
import pytest

NB, BLOCK = 32, 128


def _panel(A, piv, k, nb):
    n = A.shape[0]
    for c in range(nb):
        col = k + c
        p = col + int(np.argmax(np.abs(A[col:, col]) ** 2))  # first of equal maxima
        piv[col] = p
        if p != col:
            A[[col, p], k:k + nb] = A[[p, col], k:k + nb]
        A[col + 1:, col] /= A[col, col]
        A[col + 1:, col + 1:k + nb] -= np.outer(A[col + 1:, col], A[col, col + 1:k + nb])


def _swap(A, piv, cols, k, nb):
    for c in range(nb):
        r, p = k + c, piv[k + c]
        if p != r and len(cols):
            A[np.ix_([r, p], cols)] = A[np.ix_([p, r], cols)]


def _trsm(A, k, nb, jlo, jhi):
    L = np.tril(A[k:k + nb, k:k + nb], -1) + np.eye(nb)
    A[k:k + nb, jlo:jhi] = np.linalg.solve(L, A[k:k + nb, jlo:jhi])


def _unblocked(A):
    n = A.shape[0]
    piv = np.zeros(n, dtype=int)
    for k in range(0, n, NB):
        nb = min(NB, n - k)
        _panel(A, piv, k, nb)
        _swap(A, piv, [j for j in range(n) if not k <= j < k + nb], k, nb)
        if k + nb < n:
            _trsm(A, k, nb, k + nb, n)
            A[k + nb:, k + nb:] -= A[k + nb:, k:k + nb] @ A[k:k + nb, k + nb:]
    return piv


def _blocked(A):
    n = A.shape[0]
    piv = np.zeros(n, dtype=int)
    for K in range(0, n, BLOCK):
        KE = min(K + BLOCK, n)
        for k in range(K, KE, NB):
            nb = min(NB, KE - k)
            kn = k + nb
            _panel(A, piv, k, nb)
            _swap(A, piv, [j for j in range(K, KE) if not k <= j < kn], k, nb)
            if kn < KE:
                _trsm(A, k, nb, kn, KE)
                A[kn:, kn:KE] -= A[kn:, k:kn] @ A[k:kn, kn:KE]
        _swap(A, piv, [j for j in range(n) if not K <= j < KE], K, KE - K)
        if KE < n:
            for k in range(K, KE, NB):
                nb = min(NB, KE - k)
                kn = k + nb
                _trsm(A, k, nb, KE, n)
                A[kn:KE, KE:] -= A[kn:KE, k:kn] @ A[k:kn, KE:]
            A[KE:, KE:] -= A[KE:, K:KE] @ A[K:KE, KE:]
    return piv


def _residual(A0, LU, piv):
    n = A0.shape[0]
    PA = A0.copy()
    for r in range(n):
        PA[[r, piv[r]]] = PA[[piv[r], r]]
    L = np.tril(LU, -1) + np.eye(n)
    return np.max(np.abs(PA - L @ np.triu(LU))) / np.max(np.abs(A0))


@pytest.mark.parametrize("n", [40, 128, 129, 257, 450])
def test_blocked_order_factors_with_the_unblocked_pivots(n):
    rng = np.random.default_rng(n)
    A0 = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Au, Ab = A0.copy(), A0.copy()
    pu, pb = _unblocked(Au), _blocked(Ab)
    assert np.array_equal(pu, pb)
    assert _residual(A0, Ab, pb) < 1e-12
    assert np.max(np.abs(Au - Ab)) < 1e-9 * np.max(np.abs(Au))

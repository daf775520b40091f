"""The plain form's FP64 LU schedule (csrc/dense.cu) restated in numpy.

nalgebra's partial-pivot LU (solve.rs:166-171 -> nalgebra lu(): at column c
the first row maximising |re| + |im| is swapped with row c across the whole
matrix, then the column is scaled and the trailing part updated).  The device
code factors panels of 32 columns: inside a panel the swaps touch only the
panel's columns and the other columns take the panel's swaps together
afterwards, then the row block U12 and the trailing GEMM.  These tests check,
on the CPU, that deferring the swaps changes nothing (bit for bit against the
same panel schedule with whole-row swaps) and that the pivots and factors
match the unblocked algorithm."""
import numpy as np
import pytest

NB = 32


def icamax(col):
    v = np.abs(col.real) + np.abs(col.imag)
    return int(np.argmax(v))  # first maximum


def lu_unblocked(A):
    A = A.copy()
    n = A.shape[0]
    piv = np.zeros(n, dtype=np.int64)
    for c in range(n):
        p = c + icamax(A[c:, c])
        piv[c] = p
        if p != c:
            A[[c, p], :] = A[[p, c], :]
        d = A[c, c]
        if d != 0:
            A[c + 1:, c] *= 1.0 / d
            A[c + 1:, c + 1:] -= np.outer(A[c + 1:, c], A[c, c + 1:])
    return A, piv


def lu_panels(A, defer):
    """Panels of NB columns; `defer`: swaps inside the panel only, the rest
    applied after the panel (the device schedule), else whole-row swaps."""
    A = A.copy()
    n = A.shape[0]
    piv = np.zeros(n, dtype=np.int64)
    for p0 in range(0, n, NB):
        pend = min(p0 + NB, n)
        for c in range(p0, pend):
            p = c + icamax(A[c:, c])
            piv[c] = p
            if p != c:
                cols = slice(p0, pend) if defer else slice(0, n)
                A[[c, p], cols] = A[[p, c], cols]
            d = A[c, c]
            if d != 0:
                inv = 1.0 / d
                A[c + 1:, c] = A[c + 1:, c] * inv
                for j in range(c + 1, pend):
                    A[c + 1:, j] -= A[c + 1:, c] * A[c, j]
        if defer:
            outside = [j for j in range(n) if not p0 <= j < pend]
            for c in range(p0, pend):
                p = piv[c]
                if p != c:
                    t = A[c, outside].copy()
                    A[c, outside] = A[p, outside]
                    A[p, outside] = t
        if pend < n:
            L11 = np.tril(A[p0:pend, p0:pend], -1) + np.eye(pend - p0)
            A[p0:pend, pend:] = np.linalg.solve(L11, A[p0:pend, pend:])
            A[pend:, pend:] -= A[pend:, p0:pend] @ A[p0:pend, pend:]
    return A, piv


def _matrix(n, seed, ties=False):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    if ties:
        # equal |re| + |im| down whole columns: the first maximum must win
        A = np.round(A)
        A[:, ::3] = (1 + 1j) * np.sign(rng.normal(size=(n, (n + 2) // 3)))
    return A


@pytest.mark.parametrize("n,seed,ties", [(1, 0, False), (31, 1, False), (32, 2, False), (33, 3, False),
                                         (100, 4, False), (97, 5, True), (130, 6, True)])
def test_deferred_swaps_change_nothing(n, seed, ties):
    A = _matrix(n, seed, ties)
    F1, p1 = lu_panels(A, defer=False)
    F2, p2 = lu_panels(A, defer=True)
    assert np.array_equal(p1, p2)
    assert np.array_equal(F1, F2)


@pytest.mark.parametrize("n,seed", [(33, 7), (100, 8), (129, 9)])
def test_panels_match_unblocked(n, seed):
    A = _matrix(n, seed)
    F0, p0 = lu_unblocked(A)
    F2, p2 = lu_panels(A, defer=True)
    assert np.array_equal(p0, p2)
    assert np.max(np.abs(F2 - F0)) <= 1e-11 * np.max(np.abs(F0))
    # P A = L U
    L = np.tril(F2, -1) + np.eye(n)
    U = np.triu(F2)
    PA = A.copy()
    for c in range(n):
        PA[[c, p2[c]], :] = PA[[p2[c], c], :]
    assert np.linalg.norm(L @ U - PA) <= 1e-12 * np.linalg.norm(A)


def test_zero_column_is_skipped():
    A = np.eye(5, dtype=np.complex128)
    A[:, 2] = 0
    F, p = lu_panels(A, defer=True)
    assert p[2] == 2 and np.all(F[:, 2] == 0)

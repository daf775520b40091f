"""Host-side restatements (numpy, CPU) of the LU preconditioner's schedule in
csrc/lu32.cu: the grouped delayed trailing update, the diagonal-block
elimination sweep that yields L11^-1 and U11^-1 together, and the ticket order
of the one-launch block substitution.  They check the algebra and the region
bookkeeping of the launch plan at small block sizes; the device kernels are
checked against FP64 LU in tests/test_gpu_lu.py."""
import numpy as np
import pytest


def _matrix(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return a + 2 * n * np.eye(n)  # no pivoting needed


def _lu_unblocked(a):
    a = a.copy()
    n = len(a)
    for j in range(n):
        a[j + 1:, j] /= a[j, j]
        a[j + 1:, j + 1:] -= np.outer(a[j + 1:, j], a[j, j + 1:])
    return a


def _lu_grouped(a, lb, group):
    """The launch plan of lu_precond_setup: for each group of `group` block
    steps starting at k, step k + j (j > 0) first receives the updates of steps
    k .. k + j - 1 on its block column (from the diagonal block down) and its
    block row; then its diagonal block and panels; after the group one update
    of the rest with every step's panels."""
    a = a.copy()
    n = len(a)
    nblk = (n + lb - 1) // lb
    for k in range(0, nblk, group):
        panels = []  # (rows, L21 over those rows, cols, U12 over those cols) per step
        for j in range(group):
            st = k + j
            if st >= nblk:
                break
            c0 = st * lb
            c1 = min(c0 + lb, n)
            for (r0, l21, q0, u12) in panels:
                # block column st from its diagonal block down, and block row st
                a[c0:, c0:c1] -= l21[c0 - r0:] @ u12[:, c0 - q0:c1 - q0]
                a[c0:c1, c1:] -= l21[c0 - r0:c1 - r0] @ u12[:, c1 - q0:]
            d = _lu_unblocked(a[c0:c1, c0:c1])
            a[c0:c1, c0:c1] = d
            if c1 >= n:
                break
            l11 = np.tril(d, -1) + np.eye(c1 - c0)
            u11 = np.triu(d)
            a[c1:, c0:c1] = a[c1:, c0:c1] @ np.linalg.inv(u11)   # L21 = A21 U11^-1
            a[c0:c1, c1:] = np.linalg.inv(l11) @ a[c0:c1, c1:]   # U12 = L11^-1 A12
            panels.append((c1, a[c1:, c0:c1].copy(), c1, a[c0:c1, c1:].copy()))
        r = (k + group) * lb
        for (r0, l21, q0, u12) in panels:
            if r < n:
                a[r:, r:] -= l21[r - r0:] @ u12[:, r - q0:]
    return a


@pytest.mark.parametrize("n", [13, 16, 30, 37, 64])
@pytest.mark.parametrize("group", [1, 2, 4])
def test_grouped_delayed_update_matches_lu(n, group):
    a = _matrix(n, n + group)
    ref = _lu_unblocked(a)
    got = _lu_grouped(a, 4, group)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def _diag_sweep(a):
    """lu_diag_kernel's elimination: Z ends as L^-1 (strictly lower, unit
    diagonal implied) + U^-1 (upper) of A = L U without pivoting."""
    z = a.astype(complex).copy()
    n = len(z)
    idx = np.arange(n)
    for j in range(n):
        col, row = z[:, j].copy(), z[j, :].copy()
        pinv = 1.0 / row[j]
        cvs = col * pinv                      # row multipliers c_i / p
        cvs[j] = 1.0 + pinv                   # row j: r_c -> -r_c / p right of the pivot
        below = idx > j
        right = (idx > j).astype(float)
        for i in range(n):
            r = row.copy()
            r[j] = 0.0
            if not below[i]:
                r = r * right                 # rows at or above j: columns right of j only
            z[i] -= cvs[i] * r
        z[:, j] = np.where(idx > j, -col * pinv, col * pinv)
        z[j, j] = pinv
    return z


def test_diag_sweep_gives_both_inverses():
    a = _matrix(23, 5)
    lu = _lu_unblocked(a)
    linv = np.linalg.inv(np.tril(lu, -1) + np.eye(23))
    uinv = np.linalg.inv(np.triu(lu))
    z = _diag_sweep(a)
    assert np.abs(np.tril(z, -1) - np.tril(linv, -1)).max() < 1e-13
    assert np.abs(np.triu(z) - uinv).max() < 1e-13


def test_substitution_tickets_depend_only_on_earlier_tickets():
    """lu_trsv_kernel's ticket list: forward rows by ascending block, then
    backward rows by descending block, systems interleaved.  A row may wait
    only for rows with smaller tickets, so CTAs that already hold a ticket
    make progress in any residency."""
    nblk = [5, 1, 3, 7]
    tickets = []
    for ph in (0, 1):
        for t in range(max(nblk)):
            for s, nb in enumerate(nblk):
                if t < nb:
                    tickets.append((s, ph, t if ph == 0 else nb - 1 - t))
    pos = {tk: i for i, tk in enumerate(tickets)}
    assert len(tickets) == 2 * sum(nblk)
    for (s, ph, b), i in pos.items():
        deps = [(s, 0, k) for k in range(b)] if ph == 0 else \
               [(s, 1, k) for k in range(b + 1, nblk[s])] + [(s, 0, nblk[s] - 1)]
        assert all(pos[d] < i for d in deps)

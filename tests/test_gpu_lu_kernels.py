"""The LU preconditioner's kernels checked entry by entry (csrc/lu32.cu):
lu_diag_kernel (diagonal-block inverses), lu_gemm_kernel in its three modes
(tcgen05 trailing update on FP16 operands, TF32 L21 and U12 panels) with the expand / copy
kernels around them, and lu_trsv_kernel (one-launch block substitutions, one
to four right-hand sides per operator).

bem_lu32_factor_apply runs the same factorization and application as the
mixed form's BEM_PRECOND_LU on caller-given FP32 operators and returns the
factors.  They are compared with an FP64 no-pivot LU of the same FP32
matrices: per 128 x 128 block, the relative Frobenius error of the factors
must stay at the level of an 11-bit significand (TF32 and FP16 both carry
one; the emulated TF32 algorithm gives ~1e-3; the bound is 5e-3), while a tile shifted by one row or column gives O(1) -- the
CPU test at the end plants such a shift in the expected factors and checks
that the comparison rejects it.  The substitutions are checked against the
same block recurrences evaluated in FP64 on the returned factors (FP32
products: 1e-5), and against an FP64 solve with the exact factors (TF32
level)."""
import ctypes as C

import numpy as np
import pytest
import scipy.linalg as sl

LB = 128
TOL_FACTOR = 5e-3   # block-relative Frobenius error of F and D vs FP64 LU
TOL_APPLY = 1e-5    # substitutions vs the same recurrences in FP64
TOL_SOLVE = 2e-2    # z vs an FP64 solve with the exact factors


# --------------------------------------------------------------------------
# FP64 references (numpy, CPU)

def operator(n, seed):
    """A complex matrix with the BEM operators' structure for this purpose: a
    dominant diagonal (no pivoting needed) and dense O(1/sqrt(n)) coupling, as
    FP32."""
    rng = np.random.default_rng(seed)
    r = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2 * n)
    return (3.0 * (1.0 + 0.3j) * np.eye(n) + r).astype(np.complex64)


def lu_nopivot(a):
    """Blocked FP64 LU without pivoting: L (unit lower) and U packed in one
    matrix."""
    a = np.array(a, dtype=np.complex128)
    n = len(a)
    for k0 in range(0, n, LB):
        k1 = min(k0 + LB, n)
        d = a[k0:k1, k0:k1]
        for j in range(k1 - k0):
            d[j + 1:, j] /= d[j, j]
            d[j + 1:, j + 1:] -= np.outer(d[j + 1:, j], d[j, j + 1:])
        if k1 >= n:
            break
        a[k1:, k0:k1] = sl.solve_triangular(np.triu(d), a[k1:, k0:k1].T, trans="T", lower=False).T
        a[k0:k1, k1:] = sl.solve_triangular(d, a[k0:k1, k1:], lower=True, unit_diagonal=True)
        a[k1:, k1:] -= a[k1:, k0:k1] @ a[k0:k1, k1:]
    return a


def expected_factors(a):
    """F as the kernels leave it (L21 below and U12 above the diagonal blocks,
    L_bb U_bb on them) and the per-block inverse tiles of D."""
    lu = lu_nopivot(a)
    n = len(lu)
    f = lu.copy()
    tiles = []
    for k0 in range(0, n, LB):
        k1 = min(k0 + LB, n)
        d = lu[k0:k1, k0:k1]
        lo = np.tril(d, -1) + np.eye(k1 - k0)
        up = np.triu(d)
        f[k0:k1, k0:k1] = lo @ up
        tiles.append(np.tril(np.linalg.inv(lo), -1) + np.triu(np.linalg.inv(up)))
    return lu, f, tiles


def _tf32(x):
    """FP32 values as the TF32 tensor-core path reads them (low 13 mantissa
    bits dropped)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    return (x.view(np.uint32) & np.uint32(0xFFFFE000)).view(np.float32).astype(np.float64)


def _ctf32(z):
    return _tf32(z.real) + 1j * _tf32(z.imag)


def lu_tf32_emulated(a):
    """The factorization as the kernels compute it, in numpy: FP32 storage,
    diagonal blocks eliminated in FP32, panels and trailing updates from
    TF32-truncated operands (accumulated in FP64 here, FP32 on the device).
    Its error against lu_nopivot is the error level a correct device
    factorization reaches on the same matrix."""
    a = np.array(a, dtype=np.complex64).astype(np.complex128)
    n = len(a)
    for k0 in range(0, n, LB):
        k1 = min(k0 + LB, n)
        d = a[k0:k1, k0:k1].astype(np.complex64)
        for j in range(k1 - k0):
            d[j + 1:, j] /= d[j, j]
            d[j + 1:, j + 1:] -= np.outer(d[j + 1:, j], d[j, j + 1:])
        a[k0:k1, k0:k1] = d
        if k1 >= n:
            break
        li = np.linalg.inv(np.tril(d, -1) + np.eye(k1 - k0)).astype(np.complex64)
        ui = np.linalg.inv(np.triu(d)).astype(np.complex64)
        l21 = (_ctf32(a[k1:, k0:k1]) @ _ctf32(ui)).astype(np.complex64)
        u12 = (_ctf32(li) @ _ctf32(a[k0:k1, k1:])).astype(np.complex64)
        a[k1:, k0:k1] = l21
        a[k0:k1, k1:] = u12
        a[k1:, k1:] = (a[k1:, k1:] - _ctf32(l21) @ _ctf32(u12)).astype(np.complex64)
    return a


def block_errors(got, ref):
    """Relative Frobenius error of every 128 x 128 block (blocks of ref that
    are zero are compared in absolute terms against the matrix norm)."""
    n = ref.shape[0]
    scale = np.linalg.norm(ref) / max(1, (n + LB - 1) // LB)
    worst = 0.0
    for i in range(0, n, LB):
        for j in range(0, ref.shape[1], LB):
            r = ref[i:i + LB, j:j + LB]
            g = got[i:i + LB, j:j + LB]
            den = max(np.linalg.norm(r), 1e-3 * scale)
            worst = max(worst, np.linalg.norm(g - r) / den)
    return worst


def apply_with(f, tiles, q):
    """lu_trsv_kernel's recurrences in FP64 on given factors:
    forward  y = q_b - sum_{k<b} L_bk z_k,  z_b = y + strict_lower(D_b) y;
    backward w = z_b - sum_{k>b} U_bk z_k,  z_b = upper(D_b) w."""
    n = len(f)
    nb = (n + LB - 1) // LB
    z = np.array(q, dtype=np.complex128)
    for b in range(nb):
        r0, r1 = b * LB, min(b * LB + LB, n)
        y = z[r0:r1] - f[r0:r1, :r0] @ z[:r0]
        z[r0:r1] = y + np.tril(tiles[b], -1) @ y
    for b in reversed(range(nb)):
        r0, r1 = b * LB, min(b * LB + LB, n)
        w = z[r0:r1] - f[r0:r1, r1:] @ z[r1:]
        z[r0:r1] = np.triu(tiles[b]) @ w
    return z


# --------------------------------------------------------------------------
# the device side, through the C ABI

def _pad64(n):
    return (n + 63) // 64 * 64


def factor_apply(ctx, mats, rhs_per_op, seed=0):
    """Factors the operators `mats` (each shared by rhs_per_op[i] systems)
    and applies M to one random vector per system.  Returns per operator
    (F, D tiles, [(q, z) per right-hand side]) and the replaced-pivot count."""
    ns, lds, offs, qs = [], [], [], []
    off = 0
    rng = np.random.default_rng(seed)
    blocks = []
    for a, r in zip(mats, rhs_per_op):
        n = len(a)
        ld = _pad64(n)
        blocks.append((off, ld, n))
        for _ in range(r):
            ns.append(n)
            lds.append(ld)
            offs.append(off)
            qs.append(rng.standard_normal(n) + 1j * rng.standard_normal(n))
        off += ld * n
    A = np.zeros(off, dtype=np.complex64)
    for (o, ld, n), a in zip(blocks, mats):
        col = np.zeros((n, ld), dtype=np.complex64)  # column-major: row j of col = column j
        col[:, :n] = a.T
        A[o:o + ld * n] = col.reshape(-1)
    F = np.zeros_like(A)
    d_entries = sum(((n + LB - 1) // LB) * LB * LB for (_, _, n) in blocks)
    D = np.zeros(d_entries, dtype=np.complex64)
    q = np.concatenate(qs).astype(np.complex128)
    z = np.zeros_like(q)
    piv = C.c_int(0)
    arr = lambda v: (C.c_int64 * len(v))(*v)
    import cc_abstemious_gb300 as bem
    st = ctx.lib.bem_lu32_factor_apply(ctx.h, len(ns), arr(ns), arr(lds), arr(offs), len(A),
                                       bem._ptr(A), bem._ptr(F), bem._ptr(D), d_entries, bem._ptr(q),
                                       bem._ptr(z), C.byref(piv))
    assert st == 0, ctx.lib.bem_last_error(ctx.h)
    out, v, dpos = [], 0, 0
    for (o, ld, n), r in zip(blocks, rhs_per_op):
        f = F[o:o + ld * n].reshape(n, ld)[:, :n].T.astype(np.complex128)
        nb = (n + LB - 1) // LB
        # the tile of a partial last block holds its nb x nb corner only
        tiles = [D[dpos + b * LB * LB:dpos + (b + 1) * LB * LB].reshape(LB, LB).T.astype(np.complex128)
                 [:min(LB, n - b * LB), :min(LB, n - b * LB)] for b in range(nb)]
        dpos += nb * LB * LB
        pairs = []
        for _ in range(r):
            pairs.append((q[v:v + n], z[v:v + n]))
            v += n
        out.append((f, tiles, pairs))
    return out, piv.value


def check_operator(a, f, tiles, pairs):
    lu, f_ref, tiles_ref = expected_factors(a)
    ef = block_errors(f, f_ref)
    ed = max(block_errors(t, r) for t, r in zip(tiles, tiles_ref))
    # the bound: TOL_FACTOR, or three times what the emulated TF32
    # factorization of the same matrix reaches where that is larger (operators
    # whose blocks come out of cancellation)
    emu = lu_tf32_emulated(a)
    f_emu = emu.copy()
    for k0 in range(0, len(a), LB):
        k1 = min(k0 + LB, len(a))
        d = emu[k0:k1, k0:k1]
        f_emu[k0:k1, k0:k1] = (np.tril(d, -1) + np.eye(k1 - k0)) @ np.triu(d)
    bound = max(TOL_FACTOR, 3.0 * block_errors(f_emu, f_ref))
    print("factor error %.3g, inverse-tile error %.3g, bound %.3g" % (ef, ed, bound))
    assert ef <= bound, ("factors", ef, bound)
    assert ed <= bound, ("diagonal-block inverses", ed, bound)
    lo = np.tril(lu, -1) + np.eye(len(lu))
    up = np.triu(lu)
    for q, z in pairs:
        z_rec = apply_with(f, tiles, q)
        assert np.linalg.norm(z - z_rec) <= TOL_APPLY * np.linalg.norm(z_rec), "substitution recurrences"
        z_lu = sl.solve_triangular(up, sl.solve_triangular(lo, q, lower=True, unit_diagonal=True))
        assert np.linalg.norm(z - z_lu) <= TOL_SOLVE * np.linalg.norm(z_lu), "FP64 solve"
    return ef, ed


# --------------------------------------------------------------------------

@pytest.fixture(scope="module")
def ctx():
    bem = pytest.importorskip("cc_abstemious_gb300")
    return bem.Context.default()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [100, 128, 300, 512, 640, 768, 1100])
def test_factors_single_operator(ctx, n):
    """One partial block (100), exactly one block (128), a group of three
    steps with a partial last block (300), one full group (512), groups of
    4 + 1 (640) and 4 + 2 (768) steps, and 4 + 4 + 1 with a partial block
    (1100)."""
    a = operator(n, n)
    (res,), piv = factor_apply(ctx, [a], [1])
    assert piv == 0
    check_operator(a, *res)


@pytest.mark.gpu
@pytest.mark.parametrize("group", [4, 8])
def test_factors_step_groups_of_eight(ctx, group):
    """Systems from 4096 unknowns on may take eight block steps per pass over
    A22 (K = 2048): 4600 unknowns (36 blocks, the last partial: groups of
    8 + 8 + 8 + 8 + 4) factored with both group sizes, through the tuning
    table's override."""
    n = 4600
    a = operator(n, 5)
    ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"group", group))
    try:
        (res,), piv = factor_apply(ctx, [a], [2], seed=9)
    finally:
        ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"group", -1))
    assert piv == 0
    check_operator(a, *res)


@pytest.mark.gpu
def test_factors_ragged_batch_with_shared_operators(ctx):
    """Systems of different sizes factored together (all advance block step k
    at once), with groups of 1, 2, 3 and 4 right-hand sides per operator (the
    substitution tickets carry up to four vectors)."""
    sizes = [64, 130, 515, 1000, 257]
    rhs = [1, 2, 4, 1, 3]
    mats = [operator(n, 7 + n) for n in sizes]
    res, piv = factor_apply(ctx, mats, rhs, seed=3)
    assert piv == 0
    for a, r in zip(mats, res):
        check_operator(a, *r)


@pytest.mark.gpu
def test_factors_bem_operator(ctx):
    """A Burton-Miller operator of the library itself (icosphere of 1280
    triangles, ka = 3), as the mixed form assembles it in FP32."""
    import os
    import tempfile
    import cc_abstemious_gb300 as bem
    from cc_abstemious_gb300 import meshgen, workloads
    wd = tempfile.mkdtemp(prefix="bem_lu_k_")
    nodes, tris = meshgen.icosphere(3)
    path = os.path.join(wd, "ico3.vtk")
    meshgen.write_vtk(path, nodes, tris, 5)
    inp = workloads.base_input(path, [3.0 * 343.0 / (2 * np.pi)], method="BurtonMiller",
                               solver={"Iterative": {"tolerance": 1e-9, "max_iterations": 1000}})
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    n = pd.n
    buf = np.zeros(2 * n * n, dtype=np.float32)
    ctx.check(ctx.lib.bem_get_system_matrix_fp32(ctx.h, pd.h, bem._ptr(buf), n))
    a = (buf[0::2] + 1j * buf[1::2]).reshape(n, n).T.astype(np.complex64)
    (res,), piv = factor_apply(ctx, [a], [2], seed=11)
    assert piv == 0
    check_operator(a, *res)


def test_comparison_rejects_shifted_tile():
    """CPU: the comparison used above fails on factors with one tile shifted
    by a row or a column (planted in the expected values, not on the GPU)."""
    a = operator(300, 1)
    lu, f, tiles = expected_factors(a)
    assert block_errors(f, f) == 0.0
    for shift in ((1, 0), (0, 1)):
        g = f.copy()
        blk = g[128:256, 0:128]
        g[128:256, 0:128] = np.roll(blk, shift, axis=(0, 1))
        assert block_errors(g, f) > 20 * TOL_FACTOR
    t = [x.copy() for x in tiles]
    t[1] = np.roll(t[1], 1, axis=1)
    assert max(block_errors(x, r) for x, r in zip(t, tiles)) > 20 * TOL_FACTOR
    q = np.ones(300, dtype=complex)
    z_ok = apply_with(f, tiles, q)
    z_bad = apply_with(f, t, q)
    assert np.linalg.norm(z_bad - z_ok) > 100 * TOL_APPLY * np.linalg.norm(z_ok)

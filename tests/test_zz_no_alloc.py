"""bem_gmres_solve_noalloc: the dense GMRES entry point for callers that cannot
allocate device memory at solve time (their device memory is handed to their
own pool up front, or they run under a fixed memory budget).  Its working
memory is a fixed array inside the library, so each call only launches kernels.

The checks: called through the C ABI with device buffers, calls in a row of
growing size (each runs over the previous call's leftovers, and a hidden
allocation that grows with n would show on the later, larger calls) give the
same answer and mat-vec count as bem_gmres_solve; the calls after the first
leave the device's free memory unchanged; a size beyond the array is refused up
front.  This file is collected last so a failure here comes after every other
test.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

bem = pytest.importorskip("cc_abstemious_gb300")
torch = pytest.importorskip("torch")


def _device_matrix(A):
    # column-major A == row-major storage of A^T
    return torch.from_numpy(np.ascontiguousarray(np.asarray(A, dtype=np.complex128).T)).cuda()


def _noalloc(ctx, Ad, bd, n, max_it, tol):
    rep = bem.SolveReport()
    st = ctx.lib.bem_gmres_solve_noalloc(ctx.h, n, C.c_void_p(Ad.data_ptr()), n, max_it, tol,
                                         C.c_void_p(bd.data_ptr()), C.byref(rep))
    return st, rep


def test_noalloc_matches_gmres_calls_in_a_row():
    ctx = bem.Context.default()
    # the reference's golden system first, then larger ones (n = 4096 is the
    # stated limit at any iteration count)
    cases = [(100, 10, 100, 1e-8), (300, 3, 300, 1e-10), (4096, 7, 4096, 1e-10)]
    free = []
    for i, (n, seed, max_it, tol) in enumerate(cases):
        A, b = O.generate_random_ab(n, n, seed)
        Ad = _device_matrix(A)
        xd = torch.from_numpy(np.ascontiguousarray(b)).cuda()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st, rep = _noalloc(ctx, Ad, xd, n, max_it, tol)
        torch.cuda.synchronize()
        free.append((free_before, torch.cuda.mem_get_info()[0]))
        assert st == 0, ctx.lib.bem_last_error(ctx.h)
        x_ref, rep_ref = bem.gmres(A, b, max_it, tol, ctx=ctx)
        x = xd.cpu().numpy()
        assert rep.num_mv == rep_ref["num_mv"] and rep.flag == 1
        assert rep.seconds > 0.0
        assert np.max(np.abs(x - x_ref)) <= 1e-12 * np.max(np.abs(x_ref))
        if i == 0:
            # the golden value of src/solve.rs:220-228 (1e-6)
            assert abs(x[0] - (0.0035386336544537098 + 0.0017794290945383035j)) < 1e-6
        del Ad, xd
    # the first call on a device resolves the array's address (and may load the
    # library's device image); the later, larger calls must not change free memory
    for before, after in free[1:]:
        assert before == after, free


def test_noalloc_rejects_oversized_problem():
    ctx = bem.Context.default()
    n = 8192  # restart length 91 -> about 12 MB of workspace, beyond the fixed 8 MiB
    Ad = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
    xd = torch.ones(n, dtype=torch.complex128, device="cuda")
    st, rep = _noalloc(ctx, Ad, xd, n, n, 1e-8)
    assert st == 1
    assert b"fixed scratch" in ctx.lib.bem_last_error(ctx.h)
    assert torch.all(xd == 1)  # nothing was issued

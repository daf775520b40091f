"""Several bodies in one batch (bem_run_batch): bodies of different sizes and
boundary conditions assembled by one multi-body launch and solved by one
batched GMRES over systems of different sizes.  Each body's results must match
its one-body mixed run (same arithmetic per system) and an FP64 LU of the
same operator to 1e-6."""
import ctypes as C
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

bem = pytest.importorskip("cc_abstemious_gb300")
from cc_abstemious_gb300 import workloads  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


@pytest.fixture(scope="module")
def bodies():
    wd = tempfile.mkdtemp(prefix="bem_batch_")
    # tolerance 1e-8 on the backward error keeps the forward error against
    # FP64 LU below 1e-6 for these operators (condition numbers ~10-100)
    inps = [workloads.perturbed_sphere_input(wd, 40 + i, t, [1.0, 3.0, 5.5], tol=1e-8)
            for i, t in enumerate((900, 320, 610, 1200, 450))]
    # a body with a non-zero boundary value (the one-body assembly with the
    # right-hand-side row sums) and a first-kind body (classical, pressure:
    # FP64 operator, solved on its own)
    nv = workloads.perturbed_sphere_input(wd, 60, 500, [2.0, 4.0], tol=1e-8)
    nv["surface_bc"] = {"bc_type": "NormalVelocity", "value": [1.0, 0.5]}
    fk = workloads.perturbed_sphere_input(wd, 61, 400, [1.5], tol=1e-8)
    fk["method_type"] = "Classical"
    fk["surface_bc"] = {"bc_type": "Pressure", "value": [0.0, 0.0]}
    return inps + [nv, fk]


def _single(ctx, inp, precond=None):
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form="mixed", precond=precond, check_vs_lu=False)
    return a


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("precond", [None, "block_jacobi"])
def test_batch_matches_single_and_lu(ctx, bodies, precond):
    pds = [bem.PreData.from_dict(d, ctx=ctx) for d in bodies]
    out = bem.run_batch(pds, precond=precond, check_vs_lu=True, ctx=ctx)
    assert len(out) == len(bodies)
    for inp, (res, reps) in zip(bodies, out):
        single = _single(ctx, inp, precond)
        for r, s, rep, srep in zip(res, single.results, reps, single.reports):
            assert rep["flag"] == 1
            assert 0 <= rep["rel_err_vs_lu"] < 1e-6, rep
            assert rep["iterations"] == srep["iterations"]
            # the multi-body assembly kernel (parameters staged in shared
            # memory) may contract a few FP32 products into FMAs differently
            # from the one-body kernel; a last-bit change of the operator moves
            # the GMRES iterate within its tolerance, far below 1e-6
            assert _rel(r.scattered, s.scattered) <= 1e-7
            assert _rel(r.incident, s.incident) <= 1e-14
            if precond:
                assert rep["precond"] == bem.PRECOND_BLOCK_JACOBI or inp["method_type"] == "Classical"


def test_batch_chunks(ctx, bodies):
    """Operators bounded to about two bodies at a time: same results as one chunk."""
    pds = [bem.PreData.from_dict(d, ctx=ctx) for d in bodies[:5]]
    whole = bem.run_batch(pds, ctx=ctx)
    chunked = bem.run_batch(pds, max_operator_bytes=3 * 1024 * 1024 * 8 * 3, ctx=ctx)
    for (rw, pw), (rc, pc) in zip(whole, chunked):
        for a, b in zip(rw, rc):
            assert np.array_equal(a.scattered, b.scattered)
        assert [p["iterations"] for p in pw] == [p["iterations"] for p in pc]


def test_batch_errors(ctx, bodies):
    lib = ctx.lib
    assert lib.bem_run_batch(ctx.h, None, 1, 0, None, None, None, 0, 0) == 1
    handles = (C.c_void_p * 1)()
    assert lib.bem_run_batch(ctx.h, handles, 1, 0, None, None, None, 0, 0) == 1  # null problem
    pd = bem.PreData.from_dict(bodies[1], ctx=ctx)
    handles[0] = pd.h
    assert lib.bem_run_batch(ctx.h, handles, 1, 0, None, None, None, 0, -1) == 1
    assert lib.bem_run_batch(ctx.h, handles, 0, 0, None, None, None, 0, 0) == 0
    # outputs are optional
    assert lib.bem_run_batch(ctx.h, handles, 1, 0, None, None, None, 0, 0) == 0

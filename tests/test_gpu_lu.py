"""LU preconditioner of the mixed form: FP32 operators factored without
pivoting (tensor-core panel and FP16 trailing updates), applied by blocked triangular
solves inside the FP64 GMRES.  The answer is decided by the FP64 residual, so
the checks are: every solve within 1e-6 of an FP64 LU, and far fewer
iterations than without a preconditioner."""
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

bem = pytest.importorskip("cc_abstemious_gb300")
from cc_abstemious_gb300 import meshgen, workloads  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


@pytest.fixture(scope="module")
def wd():
    return tempfile.mkdtemp(prefix="bem_lu_")


def _run(ctx, inp, precond):
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form="mixed", precond=precond, check_vs_lu=True)
    return a.reports


def _icosphere_input(wd, sub, ka, method="BurtonMiller"):
    nodes, tris = meshgen.icosphere(sub)
    path = os.path.join(wd, "ico%d.vtk" % sub)
    meshgen.write_vtk(path, nodes, tris, 5)
    return workloads.base_input(path, [ka * 343.0 / (2 * np.pi)], method=method,
                                solver={"Iterative": {"tolerance": 1e-9, "max_iterations": 1000}})


@pytest.mark.parametrize("sub,method", [(1, "BurtonMiller"), (2, "BurtonMiller"), (3, "Classical")])
def test_lu_small_and_block_multiples(ctx, wd, sub, method):
    """80 unknowns (one partial block, no trailing update), 320, and 1280 (a
    multiple of the block size)."""
    inp = _icosphere_input(wd, sub, 2.0, method)
    r0 = _run(ctx, inp, None)
    r1 = _run(ctx, inp, "lu")
    for a, b in zip(r0, r1):
        assert b["flag"] == 1 and b["precond"] == bem.PRECOND_LU
        assert 0 <= b["rel_err_vs_lu"] < 1e-6, b
        assert b["iterations"] <= max(4, a["iterations"] // 2), (a["iterations"], b["iterations"])


@pytest.mark.parametrize("ntri", [128, 130, 256, 258])
def test_lu_block_edges(ctx, wd, ntri):
    """Exactly one and two blocks of 128 (no panels after the last), and one
    unknown past them (a 2-unknown last block)."""
    inp = workloads.perturbed_sphere_input(wd, 50 + ntri, ntri, [1.5, 4.0], tol=1e-10)
    r1 = _run(ctx, inp, "lu")
    for b in r1:
        assert b["flag"] == 1 and b["precond"] == bem.PRECOND_LU
        assert 0 <= b["rel_err_vs_lu"] < 1e-6, b
        assert b["iterations"] <= 8


def test_lu_hard_impedance(ctx, wd):
    """Impedance condition at high ka, where unpreconditioned GMRES(32) needs
    hundreds of iterations."""
    inp = workloads.perturbed_sphere_input(wd, 5, 1500, [3.0, 8.0, 12.0], tol=1e-8)
    r0 = _run(ctx, inp, None)
    r1 = _run(ctx, inp, "lu")
    for a, b in zip(r0, r1):
        assert b["flag"] == 1 and b["precond"] == bem.PRECOND_LU
        assert 0 <= b["rel_err_vs_lu"] < 1e-6, b
        assert b["iterations"] < a["iterations"]
    print("iterations none / lu:", [r["iterations"] for r in r0], [r["iterations"] for r in r1])
    assert max(r["iterations"] for r in r1) <= 30


def test_lu_ragged_batch(ctx, wd):
    inps = [workloads.perturbed_sphere_input(wd, 70 + i, t, [2.0, 6.0], tol=1e-8)
            for i, t in enumerate((300, 1100, 640))]
    pds = [bem.PreData.from_dict(d, ctx=ctx) for d in inps]
    out = bem.run_batch(pds, precond="lu", check_vs_lu=True, ctx=ctx)
    for inp, (res, reps) in zip(inps, out):
        single = _run(ctx, inp, "lu")
        for r, s in zip(reps, single):
            assert r["flag"] == 1 and r["precond"] == bem.PRECOND_LU
            assert 0 <= r["rel_err_vs_lu"] < 1e-6
            assert abs(r["iterations"] - s["iterations"]) <= 1


def test_lu_first_kind(ctx, wd):
    """A first-kind operator keeps an FP64 operator; the LU is built from its
    FP32 rounding."""
    inp = workloads.perturbed_sphere_input(wd, 9, 400, [1.5], tol=1e-8)
    inp["method_type"] = "Classical"
    inp["surface_bc"] = {"bc_type": "Pressure", "value": [0.0, 0.0]}
    r0 = _run(ctx, inp, None)[0]
    r = _run(ctx, inp, "lu")[0]
    assert r["flag"] == 1 and r["precond"] == bem.PRECOND_LU
    assert 0 <= r["rel_err_vs_lu"] < 1e-6
    assert r["iterations"] < r0["iterations"]


def test_refined_form(ctx, wd):
    """Operator at FP64 accuracy + tensor-core LU preconditioner: FP64-level agreement with the
    FP64 LU where the FP32 operator of the mixed form stops near 1e-7."""
    inp = workloads.perturbed_sphere_input(wd, 12, 2500, [4.0, 9.0], tol=1e-11)
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form="refined", precond="lu", check_vs_lu=True)
    m = _run(ctx, inp, "lu")
    for r, rm in zip(a.reports, m):
        assert r["flag"] == 1 and r["precond"] == bem.PRECOND_LU
        assert 0 <= r["rel_err_vs_lu"] < 1e-8, r
        assert r["rel_err_vs_lu"] < rm["rel_err_vs_lu"]
        assert r["iterations"] <= 12


def test_mixed_rounded_form(ctx, wd):
    """The mixed form over operators rounded once from their float-float
    values: within 1e-6 of FP64 LU, and closer than the mixed form over the
    single-precision assembly (whose entries carry a few FP32 ulps)."""
    inp = workloads.perturbed_sphere_input(wd, 17, 2400, [2.0, 6.0, 10.0], tol=1e-10)
    rm = _run(ctx, inp, "lu")
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form="mixed_rounded", precond="lu", check_vs_lu=True)
    e_mixed = max(r["rel_err_vs_lu"] for r in rm)
    e_round = max(r["rel_err_vs_lu"] for r in a.reports)
    for r in a.reports:
        assert r["flag"] == 1 and 0 <= r["rel_err_vs_lu"] < 1e-6, r
    assert e_round < e_mixed, (e_round, e_mixed)
    print("max error vs FP64 LU: mixed %.3g, mixed_rounded %.3g" % (e_mixed, e_round))


@pytest.mark.parametrize("precond", [None, "block_jacobi", "lu"])
def test_refined_form_reaches_fp64_level(ctx, wd, precond):
    """The refined form holds each FP64 operator as its FP32 rounding plus the
    FP32 rounding of the remainder and applies it in float-float: at a tight
    backward-error tolerance the answer agrees with the FP64 LU at FP64 level,
    which neither an FP32 operator nor an operator error of 2^-24 allows."""
    inp = workloads.perturbed_sphere_input(wd, 13, 900, [2.0, 5.0], tol=1e-12)
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form="refined", precond=precond, check_vs_lu=True)
    for r in a.reports:
        assert r["flag"] == 1, r
        assert 0 <= r["rel_err_vs_lu"] < 1e-10, r


@pytest.mark.parametrize("ntri", [700, 1030, 1300])
def test_lu_partial_step_groups(ctx, wd, ntri):
    """Block counts that end inside a group of four delayed steps: 6, 9 and
    11 blocks of 128 (the last group has 2, 1 and 3 steps)."""
    inps = [workloads.perturbed_sphere_input(wd, 90 + ntri, ntri, [2.5, 7.0], tol=1e-10)]
    r1 = _run(ctx, inps[0], "lu")
    for b in r1:
        assert b["flag"] == 1 and b["precond"] == bem.PRECOND_LU
        assert 0 <= b["rel_err_vs_lu"] < 1e-6, b
        assert b["iterations"] <= 8

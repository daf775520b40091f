"""The mixed form over H-matrix operators (Hierarchical solver, csrc/hmixed.cu):
ACA-compressed leaves repacked as FP32 in cluster order, batched mat-vec in the
FP64 GMRES.  Checked against an FP64 LU of the same FP64 H-matrix (the
reference's own operator, h_matrix.rs:236-246 to_full) at the ellipsoid's
settings (leaf 64, eta 1, ACA 1e-5), against an FP64 LU of the dense operator
when the ACA tolerance is tight, and block-Jacobi on the diagonal leaves
against no preconditioner."""
import numpy as np
import pytest
import scipy.linalg as sl

pytestmark = pytest.mark.gpu
bem = pytest.importorskip("cc_abstemious_gb300")
from cc_abstemious_gb300 import workloads  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


def _input(tmp_path, kas, aca_tol, tol=1e-10, waves=1):
    pw, ps = workloads.ellipsoid_bm(str(tmp_path), n_lon=64, n_bands=21)  # 2560 triangles
    inp = dict(pw)
    inp["frequency"] = {"List": {"values": [ka * 343.0 / (2 * np.pi * 2.0) for ka in kas]}}
    inp["solver"] = {"Hierarchical": {"tolerance": tol, "max_iterations": 4000, "leaf_size": 64, "eta": 1.0,
                                      "aca_tolerance": aca_tol}}
    if waves == 2:
        inp["additional_incident_waves"] = [ps["incident_wave"]]
    return inp


def _run(ctx, inp, precond=None, check=False):
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form="mixed", precond=precond, check_vs_lu=check)
    return a


@pytest.mark.parametrize("waves", [1, 2])
def test_matches_fp64_lu_of_the_same_hmatrix(ctx, tmp_path, waves):
    kas = [2.5, 8.0]
    inp = _input(tmp_path, kas, 1e-5, waves=waves)
    a = _run(ctx, inp, precond="block_jacobi")
    phi, _ = a.surface_solution()
    nf = len(kas)
    phi = np.asarray(phi).reshape(waves, nf, -1)
    for f in range(nf):
        for r in range(waves):
            rep = a.reports_by_rhs[r][f]
            assert rep["flag"] == 1 and rep["precond"] == bem.PRECOND_BLOCK_JACOBI, rep
        pd = bem.PreData.from_dict(inp, ctx=ctx)
        pd.set_frequency_index(f)
        A = bem.HMatrix(pd, bem.EqnSide.LHS).to_full()
        lu = sl.lu_factor(A)
        for r in range(waves):
            one = dict(inp)
            one.pop("additional_incident_waves", None)
            if r == 1:
                one["incident_wave"] = inp["additional_incident_waves"][0]
            p1 = bem.PreData.from_dict(one, ctx=ctx)
            p1.set_frequency_index(f)
            inc = bem.get_incident_surface(p1)
            x = sl.lu_solve(lu, -inc)  # rigid body: H phi = -phi_inc
            err = np.linalg.norm(phi[r, f] - x) / np.linalg.norm(x)
            assert err <= 1e-6, (f, r, err)


def test_tight_aca_matches_dense_fp64_lu(ctx, tmp_path):
    inp = _input(tmp_path, [4.0], 1e-9)
    a = _run(ctx, inp, precond="block_jacobi", check=True)
    rep = a.reports[0]
    assert rep["flag"] == 1
    assert 0 <= rep["rel_err_vs_lu"] <= 1e-6, rep


def test_block_jacobi_fewer_iterations(ctx, tmp_path):
    inp = _input(tmp_path, [6.0], 1e-5, tol=1e-8)
    none = _run(ctx, inp).reports[0]
    bj = _run(ctx, inp, precond="block_jacobi").reports[0]
    assert none["flag"] == 1 and bj["flag"] == 1
    assert bj["precond"] == bem.PRECOND_BLOCK_JACOBI
    assert bj["iterations"] < none["iterations"], (bj["iterations"], none["iterations"])

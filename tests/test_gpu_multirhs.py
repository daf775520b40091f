"""Several incident waves per input (extension key additional_incident_waves):
every wave's results must equal a separate run with that wave as the
reference's single incident_wave, in every form; the mixed and refined forms
assemble and factor each frequency once for all waves."""
import copy
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

bem = pytest.importorskip("cc_abstemious_gb300")
from cc_abstemious_gb300 import workloads  # noqa: E402

WAVES = [{"PlaneWave": {"direction": [0.0, 0.0, 1.0], "amplitude": [1.0, 0.0]}},
         {"SphericalWave": {"origin": [0.0, 0.0, 3.0], "amplitude": [0.5, 0.2]}},
         {"PlaneWave": {"direction": [1.0, 1.0, 0.0], "amplitude": [0.0, 1.0]}}]


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


@pytest.fixture(scope="module")
def base():
    wd = tempfile.mkdtemp(prefix="bem_mrhs_")
    return workloads.perturbed_sphere_input(wd, 31, 700, [2.0, 6.0], tol=1e-10)


def _multi(base):
    d = copy.deepcopy(base)
    d["incident_wave"] = WAVES[0]
    d["additional_incident_waves"] = WAVES[1:]
    return d


def _single(base, r):
    d = copy.deepcopy(base)
    d["incident_wave"] = WAVES[r]
    return d


def _run(ctx, inp, form, precond=None, check=False):
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form=form, precond=precond, check_vs_lu=check)
    return a


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_num_rhs(ctx, base):
    assert bem.PreData.from_dict(_multi(base), ctx=ctx).info["num_rhs"] == 3
    assert bem.PreData.from_dict(base, ctx=ctx).info["num_rhs"] == 1


@pytest.mark.parametrize("form,precond,tol", [("plain", None, 1e-13), ("mixed", None, 1e-10),
                                              ("mixed", "lu", 1e-10), ("refined", "lu", 1e-10)])
def test_waves_match_single_runs(ctx, base, form, precond, tol):
    m = _run(ctx, _multi(base), form, precond, check=form != "plain")
    assert len(m.results_by_rhs) == 3
    for r in range(3):
        s = _run(ctx, _single(base, r), form, precond)
        for rm, rs, rep in zip(m.results_by_rhs[r], s.results, m.reports_by_rhs[r]):
            assert _rel(rm.scattered, rs.scattered) <= tol
            assert _rel(rm.incident, rs.incident) <= 1e-14
            if form != "plain":
                assert rep["flag"] == 1
                assert 0 <= rep["rel_err_vs_lu"] < 1e-6
    phi, vn = m.surface_solution()
    assert phi.shape == (3 * 2, m.predata.n)

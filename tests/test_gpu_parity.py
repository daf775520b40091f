"""GPU parity: every entry point of libbem_gb300.so against the CPU oracle on
the reference's meshes, and the reference's published known answers.

Tolerances: the plain FP64 form must agree with the oracle to 1e-12 relative
(entry-wise, relative to the largest entry) for matrices and 1e-10 relative
for solutions; the collocation geometry is bit-identical; the mixed form must
be within 1e-6 of the FP64 LU solution.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, sphere_input
from oracle import oracle as O

pytestmark = pytest.mark.gpu

bem = pytest.importorskip("cc_abstemious_gb300")


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def problems():
    return [
        ("tri_classical", sphere_input()),
        ("tri_bm", sphere_input(method_type="BurtonMiller")),
        ("quad_bm", sphere_input("sphere_quad.vtk", body_index=2, method_type="BurtonMiller")),
        ("tri_bm_interior_spherical", sphere_input(
            method_type="BurtonMiller", problem_type="Interior",
            incident_wave={"SphericalWave": {"origin": [0.0, 0.3, 3.0], "amplitude": [0.7, -0.2]}})),
        ("tri_impedance", sphere_input(method_type="BurtonMiller",
                                       surface_bc={"bc_type": "Impedance", "value": [1500.0 * 1000.0, 300.0]})),
        ("tri_pressure", sphere_input(surface_bc={"bc_type": "Pressure", "value": [0.3, -0.1]})),
        ("quad_velocity", sphere_input("sphere_quad.vtk", body_index=2,
                                       surface_bc={"bc_type": "NormalVelocity", "value": [1.0, 0.5]})),
    ]


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


@pytest.mark.parametrize("name,inp", problems())
def test_collocation_bit_exact(ctx, name, inp):
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    assert np.array_equal(pd.get_cpts(), op.cpts)


@pytest.mark.parametrize("name,inp", problems())
def test_dense_surface_matrices(ctx, name, inp):
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    H, G = bem.get_dense_surface_matrices(pd)
    Ho, Go = op.dense_surface()
    assert rel(H, Ho) < 1e-12 and rel(G, Go) < 1e-12


@pytest.mark.parametrize("name,inp", problems()[:3])
def test_dense_surface_matrices_device(ctx, name, inp):
    torch = pytest.importorskip("torch")
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    n = pd.n
    # row-major (n, n+3) storage == column-major n x n with leading dimension n+3
    Ht = torch.empty((n, n + 3), dtype=torch.complex128, device="cuda")
    Gt = torch.empty((n, n + 3), dtype=torch.complex128, device="cuda")
    bem.get_dense_surface_matrices(pd, out=(Ht.t(), Gt.t()))
    Ho, Go = O.Problem(inp).dense_surface()
    assert rel(Ht.cpu().numpy()[:, :n].T, Ho) < 1e-12
    assert rel(Gt.cpu().numpy()[:, :n].T, Go) < 1e-12


@pytest.mark.parametrize("name,inp", problems() + [
    ("tri_bm_kr40", sphere_input(method_type="BurtonMiller", frequency={"List": {"values": [9549.0]}})),
    ("quad_bm_kr40", sphere_input("sphere_quad.vtk", body_index=2, method_type="BurtonMiller",
                                  frequency={"List": {"values": [9549.0]}}))])
def test_system_matrix_fp32(ctx, name, inp):
    """Single-precision assembly (float-float phase, Taylor sin/cos) against the
    FP64 oracle: entry errors within a few FP32 ulps of the largest entry."""
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    H, G = op.dense_surface()
    a, b = op.lhs_factors()
    ref = a * H + b * G
    A = bem.get_system_matrix_fp32(pd).astype(np.complex128)
    assert rel(A, ref) < 6e-7  # ~5 FP32 ulps of the largest entry
    # Frobenius: ~1 ulp at low k r, ~3 ulps on the hypersingular terms at k r = 40
    assert np.linalg.norm(A - ref) / np.linalg.norm(ref) < (3e-7 if "kr40" in name else 1e-7)


@pytest.mark.parametrize("name,inp", problems()[:3])
def test_row_or_column(ctx, name, inp):
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    rng = np.random.default_rng(3)
    for side in (0, 1):
        J = rng.permutation(pd.n)[:40]
        J[5] = 7  # diagonal inside the list
        r = bem.get_surface_row_or_column(pd, [7], J, side)
        assert rel(r, op.row_or_column([7], J, side)) < 1e-12
        I = rng.permutation(pd.n)[:33]
        c = bem.get_surface_row_or_column(pd, I, [11], side)
        assert rel(c, op.row_or_column(I, [11], side)) < 1e-12
    with pytest.raises(bem.BemError):
        bem.get_surface_row_or_column(pd, [1, 2], [3, 4], 1)


@pytest.mark.parametrize("name,inp", problems())
def test_incident_waves(ctx, name, inp):
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    assert rel(bem.get_incident_surface(pd), op.incident_surface()) < 1e-13
    assert rel(bem.get_incident_field(pd), op.incident_field()) < 1e-13


def test_field_matrices_and_get_field(ctx):
    inp = sphere_input(method_type="BurtonMiller", output={"o_type": "Total", "field": "Pressure", "file": "",
                                                           "field_points": [[10.0, 0, 0], [0, 3.0, 1.0],
                                                                            [-2.0, -2.0, 0.5]]})
    pd = bem.PreData.from_dict(inp, ctx=ctx)
    op = O.Problem(inp)
    M, L = bem.get_dense_field_matrices(pd)
    Mo, Lo = op.dense_field()
    assert rel(M, Mo) < 1e-12 and rel(L, Lo) < 1e-12
    rng = np.random.default_rng(0)
    phi = rng.normal(size=pd.n) + 1j * rng.normal(size=pd.n)
    vn = rng.normal(size=pd.n) + 1j * rng.normal(size=pd.n)
    inc = op.incident_field()
    ref = op.get_field(Mo, Lo, phi, vn, inc)
    assert rel(bem.get_field(pd, M, L, phi, vn, inc), ref) < 1e-12
    assert rel(bem.evaluate_field(pd, phi, vn, inc), ref) < 1e-12


def test_solve_lu_golden(ctx, goldens):
    """src/solve.rs:211-218 through the device LU."""
    A, b = O.generate_random_ab(100, 100, 10)
    x = bem.solve_lu(A, b, ctx=ctx)
    g = goldens["lu_100_seed10_x0"]["value"]
    assert abs(x[0].real - g[0]) < 1e-10 and abs(x[0].imag - g[1]) < 1e-10
    xo, _ = O.lu_solve(A, b)
    assert rel(x, xo) < 1e-12


@pytest.mark.parametrize("n", [1, 31, 32, 33, 257])
def test_solve_lu_sizes(ctx, n):
    A, b = O.generate_random_ab(n, n, n)
    x = bem.solve_lu(A, b, ctx=ctx)
    xo, _ = O.lu_solve(A, b)
    assert rel(x, xo) < 1e-12


def test_solve_lu_singular(ctx):
    A = np.zeros((4, 4), dtype=np.complex128)
    A[0, 0] = 1
    with pytest.raises(bem.BemError) as e:
        bem.solve_lu(A, np.ones(4), ctx=ctx)
    assert e.value.status == 2


def test_gmres_golden(ctx, goldens):
    """src/solve.rs:220-228: GMRES(100, 1e-8), same iteration path as the oracle."""
    A, b = O.generate_random_ab(100, 100, 10)
    x, rep = bem.gmres(A, b, 100, 1e-8, ctx=ctx)
    g = goldens["lu_100_seed10_x0"]["value"]
    assert abs(x[0].real - g[0]) < 1e-6 and abs(x[0].imag - g[1]) < 1e-6
    xo, st, orep = O.gmres_dense(A, b, 100, 1e-8)
    assert rep["num_mv"] == orep.num_mv and rep["flag"] == 1
    assert rel(x, xo) < 1e-12


def test_gmres_not_converged(ctx):
    A, b = O.generate_random_ab(60, 60, 4)
    A = A - 60 * np.eye(60)  # no longer diagonally dominant: slow convergence
    x, rep = bem.gmres(A, b, 4, 1e-14, ctx=ctx)
    xo, st, orep = O.gmres_dense(A, b, 4, 1e-14)
    assert rep["flag"] == 2 and orep.flag == 2
    assert rep["num_mv"] == orep.num_mv
    assert rel(x, xo) < 1e-10


@pytest.mark.parametrize("case,kw", [
    ("rigid_sphere_plane_wave", {}),
    ("rigid_sphere_plane_wave_iterative", {"solver": {"Iterative": {"max_iterations": 1000, "tolerance": 1e-5}}}),
    ("rigid_sphere_plane_wave_burton_miller", {"method_type": "BurtonMiller"}),
])
def test_verification_goldens(ctx, goldens, case, kw):
    """src/tests/verification.rs:95-204 through Analysis::run (plain FP64)."""
    a = bem.Analysis(ctx)
    a.set_input(sphere_input(**kw))
    a.run()
    v = a.get_result()[0].scattered[0]
    g = goldens[case]
    assert abs(v.real - g["value"][0]) < g["abs_tol"] and abs(v.imag - g["value"][1]) < g["abs_tol"]
    o = O.Problem(sphere_input(**kw)).run()[0]["scattered"][0]
    assert abs(v - o) <= 1e-10 * abs(o)


@pytest.mark.parametrize("name,inp", problems())
def test_solve_for_surface_plain(ctx, name, inp):
    for solver in ({"Direct": {}}, {"Iterative": {"max_iterations": 400, "tolerance": 1e-9}}):
        d = dict(inp, solver=solver)
        pd = bem.PreData.from_dict(d, ctx=ctx)
        op = O.Problem(d)
        rhs = op.incident_surface()
        phi, vn, rep = bem.solve_for_surface(pd, rhs)
        phio, vno, st, orep = op.solve_for_surface(rhs)
        assert rel(phi, phio) < 1e-10 and rel(vn, vno) < 1e-10
        if "Iterative" in solver:
            assert rep["num_mv"] == orep.num_mv


@pytest.mark.parametrize("name,inp", problems())
def test_analysis_run_plain_vs_oracle(ctx, name, inp):
    d = dict(inp, frequency={"LinearSpaced": {"start": 50.0, "end": 150.0, "number": 3}})
    d["output"] = dict(d["output"], field_points=[[10.0, 0, 0], [0, -4.0, 2.0]])
    a = bem.Analysis(ctx)
    a.set_input(d)
    a.run()
    ref = O.Problem(d).run()
    for r, o in zip(a.get_result(), ref):
        assert r.frequency == o["frequency"]
        assert rel(r.scattered, o["scattered"]) < 1e-10
        assert rel(r.incident, o["incident"]) < 1e-12


@pytest.mark.parametrize("name,inp", problems())
def test_analysis_run_mixed_within_1e6_of_lu(ctx, name, inp):
    d = dict(inp, frequency={"LinearSpaced": {"start": 50.0, "end": 150.0, "number": 3}},
             solver={"Iterative": {"max_iterations": 400, "tolerance": 1e-10}})
    a = bem.Analysis(ctx)
    a.set_input(d)
    a.run(form="mixed", check_vs_lu=True)
    for rep in a.reports:
        assert rep["flag"] == 1
        assert 0 <= rep["rel_err_vs_lu"] < 1e-6
    ref = O.Problem(dict(d, solver={"Direct": {}})).run()
    for r, o in zip(a.get_result(), ref):
        assert rel(r.scattered, o["scattered"]) < 1e-6


def test_input_errors(ctx):
    with pytest.raises(bem.BemError) as e:
        bem.PreData.from_json("{not json", ctx=ctx)
    assert e.value.status == 1
    d = sphere_input()
    d["body_index"] = 9
    with pytest.raises(bem.BemError):
        bem.PreData.from_dict(d, ctx=ctx)
    d = sphere_input(method_type="Hypersingular")
    with pytest.raises(bem.BemError):
        bem.PreData.from_dict(d, ctx=ctx)
    d = sphere_input()
    d["body_index"] = 3.0  # serde: usize must be an integer literal
    with pytest.raises(bem.BemError):
        bem.PreData.from_dict(d, ctx=ctx)
    with pytest.raises(bem.BemError):
        bem.PreData.from_dict(sphere_input(mesh_file="/nonexistent.vtk"), ctx=ctx)


def test_input_1_json_parses(ctx):
    """src/preprocess/input_data.rs:116-122 json_reader: body_index == 3 (mesh
    path redirected to a fixture mesh)."""
    with open(os.path.join(GOLDEN, "input_1.json")) as f:
        d = json.load(f)
    d["mesh_file"] = os.path.join(GOLDEN, "sphere.vtk")
    pd = bem.PreData.from_dict(d, ctx=ctx)
    assert pd.info["body_index"] == 3
    assert pd.info["mesh_elements"] == 336


def test_vtk_reader_large_and_malformed(ctx, tmp_path):
    """The VTK reader parses blocks of more than ~1024 rows in chunks on host
    threads: a large mesh must give the oracle's collocation bit for bit, and a
    bad row anywhere (here in the middle of a block) must be reported as bad
    input with that row's text."""
    from cc_abstemious_gb300 import meshgen
    nodes, tris = meshgen.icosphere(5)
    path = tmp_path / "ico5.vtk"
    meshgen.write_vtk(str(path), nodes, tris, 5)
    d = sphere_input(mesh_file=str(path), body_index=1)
    pd = bem.PreData.from_dict(d, ctx=ctx)
    assert np.array_equal(pd.get_cpts(), O.Problem(d).cpts)
    lines = path.read_text().splitlines()
    p0 = next(i for i, l in enumerate(lines) if l.startswith("POINTS")) + 1
    c0 = next(i for i, l in enumerate(lines) if l.startswith("CELLS")) + 1
    for row, text in ((p0 + 7000, "0.5 abc 0.25"), (c0 + 15000, "x 2 3 4")):
        bad = list(lines)
        bad[row] = text
        bpath = tmp_path / "bad.vtk"
        bpath.write_text("\n".join(bad) + "\n")
        with pytest.raises(bem.BemError) as e:
            bem.PreData.from_dict(sphere_input(mesh_file=str(bpath), body_index=1), ctx=ctx)
        assert e.value.status == 1 and text in str(e.value)
    short = tmp_path / "short.vtk"
    short.write_text("\n".join(lines[:p0 + 5000]) + "\n")
    with pytest.raises(bem.BemError) as e:
        bem.PreData.from_dict(sphere_input(mesh_file=str(short), body_index=1), ctx=ctx)
    assert e.value.status == 1

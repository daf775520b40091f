"""The CPU oracle against the reference's own known-answer tests.

Each case restates a test of cc_abstemious (cited) and checks the oracle with
the reference's tolerance.  These pins are what make the oracle trustworthy
as the reference the GPU path is compared with."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, sphere_input
from oracle import oracle as O


def test_stdrng_lu_golden(goldens):
    """src/solve.rs:211-218: LU of the seeded 100x100 system."""
    A, b = O.generate_random_ab(100, 100, 10)
    x, st = O.lu_solve(A, b)
    g = goldens["lu_100_seed10_x0"]["value"]
    assert st == 0
    assert abs(x[0].real - g[0]) < 1e-10 and abs(x[0].imag - g[1]) < 1e-10


def test_gmres_golden(goldens):
    """src/solve.rs:220-228: GMRES(100, 1e-8) on the same system, 1e-6."""
    A, b = O.generate_random_ab(100, 100, 10)
    x, st, rep = O.gmres_dense(A, b, 100, 1e-8)
    g = goldens["lu_100_seed10_x0"]["value"]
    assert st == 0 and rep.flag == 1
    assert abs(x[0].real - g[0]) < 1e-6 and abs(x[0].imag - g[1]) < 1e-6


def test_uniform_usize_range():
    r = O.StdRng(10)
    vals = [r.uniform_incl(0, 6) for _ in range(2000)]
    assert min(vals) == 0 and max(vals) == 6


@pytest.mark.parametrize("case,kw", [
    ("rigid_sphere_plane_wave", {}),
    ("rigid_sphere_plane_wave_iterative", {"solver": {"Iterative": {"max_iterations": 1000, "tolerance": 1e-5}}}),
    ("rigid_sphere_plane_wave_hmatrix", {"solver": {"Hierarchical": {"max_iterations": 1000, "tolerance": 1e-5}}}),
    ("rigid_sphere_plane_wave_burton_miller", {"method_type": "BurtonMiller"}),
])
def test_verification_goldens(goldens, case, kw):
    """src/tests/verification.rs:95-204."""
    P = O.Problem(sphere_input(**kw))
    assert P.n == 324
    res = P.run()
    v = res[0]["scattered"][0]
    g = goldens[case]
    tol = g["abs_tol"]
    assert abs(v.real - g["value"][0]) < tol
    assert abs(v.imag - g["value"][1]) < tol
    if "norm" in g:
        assert abs(abs(v) - g["norm"]) < tol


def test_vtk_reader(goldens):
    """src/preprocess/mesh_data.rs:179-187."""
    m = O.Mesh(os.path.join(GOLDEN, "sphere.vtk"))
    assert m.nelem == goldens["vtk_reader_cells"]["value"]
    assert m.nbodies == 3


def test_json_reader(goldens):
    """src/preprocess/input_data.rs:116-122."""
    with open(os.path.join(GOLDEN, "input_1.json")) as f:
        inp = json.load(f)
    assert inp["body_index"] == goldens["json_reader_body_index"]["value"]


def _grid(n, scale=1.0):
    pts = np.zeros((n * n, 3))
    t = 0
    for j in range(n):
        for k in range(n):
            pts[t] = [j * scale, k * scale, 0.0]
            t += 1
    return pts


def test_cluster_tree_diameter(goldens):
    """src/solve/h_matrix/cluster.rs:120-138 (25x25 unit grid, leaf 32)."""
    bl = O.block_list(_grid(25), 32, 4.0)
    assert abs(bl["root_diameter"] - goldens["cluster_tree_diameter"]["value"]) < 1e-2


def test_block_tree(goldens):
    """src/solve/h_matrix/block.rs:104-146."""
    pts = _grid(25)
    assert O.block_tree_path_admissible(pts, 32, 4.0, [1, 1, 1]) == 1
    bl = O.block_list(pts, 32, 4.0)
    assert bool(bl["admissible"][5]) is goldens["block_list_5_admissible"]["value"]


def _aca_matrix():
    """src/solve/aca.rs:280-299: rank-13 20x100 plus 1e-8 noise."""
    m, n = 20, 100
    a, b = O.generate_random_ab(m, n, 13)
    a = a * 1e-8
    for k in range(13):
        _, c = O.generate_random_ab(m, m, k)
        _, d = O.generate_random_ab(n, n, k + 2)
        a = a + np.outer(c, d)
    return a, b


def test_mult_aca():
    """src/solve/aca.rs:280-312."""
    a, b = _aca_matrix()
    U, V, nrm = O.aca(a, 1e-6)
    assert abs(nrm - np.linalg.norm(a)) <= 0.05 * np.linalg.norm(a)
    x1 = a @ b
    x2 = U @ (V.T @ b)
    assert np.linalg.norm(x2 - x1) / np.linalg.norm(x1) < 1e-8


def _hyperbolic(n):
    """src/solve/h_matrix.rs:255-283."""
    pts = _grid(n, 1.0 / n)
    A, b = O.generate_random_ab(n * n, n * n, 10)
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    A = (1.0 / np.maximum(1e-5, d2)).astype(np.complex128)
    return pts, A, b


def test_get_hmatrix():
    """src/solve/h_matrix.rs:300-309."""
    pts, A, b = _hyperbolic(10)
    hm = O.HMatrix(pts, 20, 4.0, 1e-4, A=A)
    eps = np.linalg.norm(hm.to_full() - A) / np.linalg.norm(A)
    assert eps < 1e-6


def test_mult_hmatrix():
    """src/solve/h_matrix.rs:310-324."""
    pts, A, b = _hyperbolic(20)
    hm = O.HMatrix(pts, 20, 4.0, 1e-4, A=A)
    x1 = A @ b
    x2 = hm.gemv(1.0 + 0j, b, 0.0 + 0j, np.zeros_like(b))
    assert np.linalg.norm(x2 - x1) / np.linalg.norm(x1) < 1e-6


def test_linspace_logspace():
    """src/tools.rs:1-24 (endpoints exact)."""
    f = O.frequency_list({"LinearSpaced": {"start": 10.0, "end": 1000.0, "number": 50}})
    assert f[0] == 10.0 and f[-1] == 1000.0 and len(f) == 50
    g = O.frequency_list({"LogSpaced": {"start": 10.0, "end": 1000.0, "number": 5}})
    assert g[0] == 10.0 and g[-1] == 1000.0 and abs(g[2] - 100.0) < 1e-9


def test_quad_area_quirk():
    """elements.rs:98-102, :168, :29: quad weight x area is 1/4 of the true area."""
    P = O.Problem(sphere_input("sphere_quad.vtk", body_index=2))
    wa = (P.cpts[:, 6] * P.cpts[:, 7]).sum()
    assert 0.7 < wa < 0.85  # true area 4 pi 0.5^2 = 3.14

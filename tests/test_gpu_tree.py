"""Cluster and block trees built on the device (csrc/tree.cu, through
bem_cluster_tree) against the oracle's sequential restatement of
cluster.rs:35-105 and block.rs:38-93 (oracle.block_list) and a numpy
restatement of the cluster recursion: the same leaf clusters, the same blocks
with the same index lists in the same depth-first order, the same
admissibility flags and root diameter, bit for bit.  Point sets with many
exact ties (grids, whose bisection planes pass through points), meshes of the
benchmark bodies, random clouds, degenerate sizes, several sets in one call,
and coincident points (an error, where the reference recurses without end)."""
import os
import tempfile

import numpy as np
import pytest

from conftest import sphere_input
from oracle import oracle as O

pytestmark = pytest.mark.gpu
bem = pytest.importorskip("cc_abstemious_gb300")
from cc_abstemious_gb300 import workloads  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


def cluster_leaves(pts, leaf):
    """cluster.rs:35-72: bisect the bounding box at the midpoint of its longest
    side (the first of equal ones), points <= gamma to the first son in their
    order; leaves depth-first."""
    out = []
    stack = [np.arange(len(pts))]
    while stack:
        idx = stack.pop()
        if len(idx) <= leaf:
            out.append(idx)
            continue
        q = pts[idx, :3]
        lo, hi = q.min(axis=0), q.max(axis=0)
        j, diff = 0, 0.0
        for d in range(3):
            if hi[d] - lo[d] > diff:
                j, diff = d, hi[d] - lo[d]
        gamma = 0.5 * (lo[j] + hi[j])
        first = q[:, j] <= gamma
        assert first.any() and not first.all()
        stack.append(idx[~first])
        stack.append(idx[first])
    return out


def _grid2(n):
    j, k = np.meshgrid(np.arange(n, dtype=float), np.arange(n, dtype=float), indexing="ij")
    return np.stack([j.ravel(), k.ravel(), np.zeros(n * n)], axis=1)


def _grid3(n):
    a = np.arange(n, dtype=float)
    x, y, z = np.meshgrid(a, a, a, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def _cpts(inp, ctx):
    return bem.PreData.from_dict(inp, ctx=ctx).get_cpts()


def _check(ctx, pts, leaf, eta):
    t = bem.cluster_tree(pts, leaf, eta, ctx=ctx)
    o = O.block_list(pts, leaf, eta)
    perm, blocks = t["perm"], t["blocks"]
    assert sorted(perm.tolist()) == list(range(len(pts)))
    # leaf clusters: consecutive ranges of perm, in the reference's order
    assert t["leaves"][0][0] == 0 and t["leaves"][-1][1] == len(pts)
    assert np.array_equal(t["leaves"][1:, 0], t["leaves"][:-1, 1])
    ref = cluster_leaves(pts, leaf)
    assert len(ref) == len(t["leaves"])
    for (a, b), r in zip(t["leaves"], ref):
        assert np.array_equal(perm[a:b], r)
    # blocks: the oracle's flattened list, index lists and flags
    assert len(blocks) == len(o["admissible"])
    rows = np.concatenate([perm[a:b] for a, b in blocks[:, 0:2]])
    cols = np.concatenate([perm[a:b] for a, b in blocks[:, 2:4]])
    assert np.array_equal(np.concatenate([[0], np.cumsum(blocks[:, 1] - blocks[:, 0])]), o["row_off"])
    assert np.array_equal(np.concatenate([[0], np.cumsum(blocks[:, 3] - blocks[:, 2])]), o["col_off"])
    assert np.array_equal(rows, o["rows"]) and np.array_equal(cols, o["cols"])
    assert np.array_equal(blocks[:, 4].astype(bool), o["admissible"].astype(bool))
    assert t["root_diameter"] == o["root_diameter"]
    return t


def test_grid_with_ties_golden_setting(ctx):
    """The 25 x 25 unit grid of cluster.rs:120-138 / block.rs:104-146 (leaf
    32, eta 4): every bisection plane passes through grid points."""
    t = _check(ctx, _grid2(25), 32, 4.0)
    assert any(b[4] for b in t["blocks"])


@pytest.mark.parametrize("leaf,eta", [(8, 1.0), (1, 2.0), (27, 0.5)])
def test_cubic_grid(ctx, leaf, eta):
    _check(ctx, _grid3(12), leaf, eta)


@pytest.mark.parametrize("leaf,eta", [(32, 4.0), (64, 1.0), (5, 2.0)])
def test_sphere_mesh(ctx, leaf, eta):
    _check(ctx, _cpts(sphere_input(), ctx), leaf, eta)


def test_random_cloud(ctx):
    rng = np.random.default_rng(3)
    pts = rng.normal(size=(5000, 3)) * np.array([3.0, 1.0, 0.2])
    _check(ctx, pts, 16, 2.0)


def test_benchmark_bodies(ctx):
    wd = tempfile.mkdtemp(prefix="bem_tree_")
    pw, _ = workloads.ellipsoid_bm(wd, n_lon=128, n_bands=41)  # 10240 triangles
    _check(ctx, _cpts(pw, ctx), 64, 1.0)
    inp = workloads.perturbed_sphere_input(wd, 7, 3000, [2.0])
    _check(ctx, _cpts(inp, ctx), 64, 2.0)
    inp = workloads.rigid_sphere_bm(wd, m=12, nfreq=1)
    _check(ctx, _cpts(inp, ctx), 32, 4.0)


@pytest.mark.parametrize("n,leaf", [(1, 1), (1, 32), (32, 32), (33, 32), (2, 1)])
def test_small_sets(ctx, n, leaf):
    rng = np.random.default_rng(n)
    _check(ctx, rng.uniform(size=(n, 3)), leaf, 2.0)


def test_stride_beyond_three(ctx):
    """Points with trailing columns (the collocation layout has 8)."""
    rng = np.random.default_rng(11)
    pts = rng.uniform(size=(700, 8))
    t = bem.cluster_tree(pts, 16, 1.5, ctx=ctx)
    u = bem.cluster_tree(np.ascontiguousarray(pts[:, :3]), 16, 1.5, ctx=ctx)
    assert np.array_equal(t["perm"], u["perm"]) and np.array_equal(t["blocks"], u["blocks"])


def test_several_sets_in_one_pass(ctx):
    rng = np.random.default_rng(5)
    sets = [_grid2(9), rng.normal(size=(1234, 3)), _cpts(sphere_input(), ctx)[:, :3].copy(),
            rng.uniform(size=(3, 3)), _grid3(5)]
    many = bem.cluster_tree(sets, 16, 2.0, ctx=ctx)
    for s, m in zip(sets, many):
        one = bem.cluster_tree(s, 16, 2.0, ctx=ctx)
        assert np.array_equal(m["perm"], one["perm"])
        assert np.array_equal(m["leaves"], one["leaves"])
        assert np.array_equal(m["blocks"], one["blocks"])
        assert m["root_diameter"] == one["root_diameter"]


def test_cluster_tree_without_blocks(ctx):
    t = bem.cluster_tree(_grid3(6), 10, None, ctx=ctx)
    assert len(t["blocks"]) == 0 and len(t["leaves"]) == len(cluster_leaves(_grid3(6), 10))


def test_coincident_points_are_an_error(ctx):
    pts = np.array([[0.0, 0.0, 0.0], [1.0, 2.0, 3.0], [1.0, 2.0, 3.0]])
    with pytest.raises(bem.BemError) as e:
        bem.cluster_tree(pts, 1, 2.0, ctx=ctx)
    assert e.value.status == 1  # BEM_ERR_BAD_INPUT
    # the context stays usable
    _check(ctx, _grid2(4), 2, 1.0)

"""Launch tuning: the trailing update's tile raster (csrc/lu32.cu raster_tile,
restated here) visits every tile of a region exactly once for any
super-block shape, and the tuning table's nearest-entry lookup.  The device
side (tuned and forced parameters giving the same factors) is in
tests/test_gpu_tuning.py."""
import itertools
import json

import pytest


def raster_tile(local, tiles_i, tiles_j, sb_r, sb_c):
    per_band = tiles_i * sb_c
    band, rem = divmod(local, per_band)
    bc = min(sb_c, tiles_j - band * sb_c)
    sr, rem2 = divmod(rem, sb_r * bc)
    br = min(sb_r, tiles_i - sr * sb_r)
    return sr * sb_r + rem2 % br, band * sb_c + rem2 // br


@pytest.mark.parametrize("tiles_i,tiles_j", [(1, 1), (3, 7), (13, 5), (40, 40), (305, 76)])
@pytest.mark.parametrize("sb", [(65535, 1), (8, 32), (4, 64), (16, 32), (8, 16), (3, 5)])
def test_raster_is_a_bijection(tiles_i, tiles_j, sb):
    seen = {raster_tile(t, tiles_i, tiles_j, *sb) for t in range(tiles_i * tiles_j)}
    assert seen == set(itertools.product(range(tiles_i), range(tiles_j)))


def test_column_order_is_the_tall_raster():
    """(sb_r >= tiles_i, sb_c = 1) is the column-after-column order."""
    for t in range(13 * 5):
        assert raster_tile(t, 13, 5, 65535, 1) == (t % 13, t // 13)


def test_committed_table_is_well_formed():
    import os
    from conftest import ROOT
    path = os.path.join(ROOT, "cc_abstemious_gb300", "tuning.json")
    if not os.path.exists(path):
        pytest.skip("no tuning table committed")
    t = json.load(open(path))
    # the parameter sets each kernel's entries may carry
    kernels = {"lu_gemm_trail": [{"sb_r", "sb_c"}, {"group"}], "gm_apply_fp32": [{"unroll"}],
               "assemble32": [{"min_ctas"}]}
    for e in t["entries"]:
        assert e["kernel"] in kernels and set(e["params"]) in kernels[e["kernel"]]
        assert e["n"] > 0 and e["nsys"] > 0
        assert e["ms"] <= min(c["ms"] for c in e["candidates"]) + 1e-9

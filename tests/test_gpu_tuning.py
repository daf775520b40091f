"""Tuning table on the device: loading, the nearest-entry lookup, overrides,
and the LU factors identical in every tile raster (the raster only reorders
independent tiles)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
bem = pytest.importorskip("cc_abstemious_gb300")
from test_gpu_lu_kernels import factor_apply, operator  # noqa: E402


def _get(ctx, kernel, param, n, nsys):
    return ctx.lib.bem_ctx_get_tuning(ctx.h, kernel.encode(), param.encode(), n, nsys)


def test_table_lookup_and_overrides(tmp_path):
    ctx = bem.Context(0)
    table = {"entries": [
        {"kernel": "lu_gemm_trail", "n": 2000, "nsys": 1, "params": {"sb_r": 4, "sb_c": 64}},
        {"kernel": "lu_gemm_trail", "n": 40000, "nsys": 1, "params": {"sb_r": 16, "sb_c": 32}},
        {"kernel": "gm_apply_fp32", "n": 6144, "nsys": 16, "params": {"unroll": 16}}]}
    p = tmp_path / "t.json"
    p.write_text(json.dumps(table))
    ctx.check(ctx.lib.bem_ctx_load_tuning(ctx.h, str(p).encode()))
    assert ctx.lib.bem_ctx_tuning_source(ctx.h) == str(p).encode()
    assert _get(ctx, "lu_gemm_trail", "sb_c", 3000, 1) == 64      # nearest: n = 2000
    assert _get(ctx, "lu_gemm_trail", "sb_c", 30000, 1) == 32     # nearest: n = 40000
    assert _get(ctx, "gm_apply_fp32", "unroll", 100, 1) == 16
    assert _get(ctx, "assemble32", "min_ctas", 6144, 16) == 3     # no entry: the default
    ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"sb_c", 7))
    assert _get(ctx, "lu_gemm_trail", "sb_c", 3000, 1) == 7
    ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"sb_c", -1))
    assert _get(ctx, "lu_gemm_trail", "sb_c", 3000, 1) == 64
    ctx.check(ctx.lib.bem_ctx_load_tuning(ctx.h, None))
    assert _get(ctx, "lu_gemm_trail", "sb_c", 3000, 1) == 32
    bad = tmp_path / "bad.json"
    bad.write_text('{"entries": [{"kernel": 3}]}')
    assert ctx.lib.bem_ctx_load_tuning(ctx.h, str(bad).encode()) == 1


@pytest.mark.parametrize("raster", [(65535, 1), (8, 32), (3, 5), (1, 1)])
def test_lu_factors_independent_of_raster(raster):
    ctx = bem.Context(0)
    a = operator(1100, 5)
    ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"sb_c", 32))
    ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"sb_r", 8))
    (ref,), _ = factor_apply(ctx, [a], [1])
    ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"sb_r", raster[0]))
    ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, b"lu_gemm_trail", b"sb_c", raster[1]))
    (got,), _ = factor_apply(ctx, [a], [1])
    # every tile computes the same sums in the same order, whatever the raster
    assert np.array_equal(got[0], ref[0])
    assert all(np.array_equal(x, y) for x, y in zip(got[1], ref[1]))

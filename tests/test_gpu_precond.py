"""Preconditioners of the mixed form: block-Jacobi and the learned near-field
correction (network kernels against the CPU restatement, training on
BEM-generated operators, iteration counts and accuracy against FP64 LU)."""
import os
import tempfile

import numpy as np
import pytest

from oracle import mlp as OM

pytestmark = pytest.mark.gpu

bem = pytest.importorskip("cc_abstemious_gb300")
from cc_abstemious_gb300 import workloads  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    return bem.Context.default()


@pytest.fixture(scope="module")
def workdir():
    return tempfile.mkdtemp(prefix="bem_pc_")


def _random_weights(seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(OM.NPARAM, dtype=np.float32)
    w[OM.OFF_W1:OM.OFF_B1] = rng.normal(0, 0.25, OM.NH * OM.NF)
    w[OM.OFF_B1:OM.OFF_W2] = rng.normal(0, 0.1, OM.NH)
    w[OM.OFF_W2:OM.OFF_B2] = rng.normal(0, 1 / np.sqrt(OM.NH), OM.NH * OM.NH)
    w[OM.OFF_B2:OM.OFF_W3] = rng.normal(0, 0.1, OM.NH)
    w[OM.OFF_W3:OM.OFF_B3] = rng.normal(0, 0.2, OM.NO * OM.NH)
    w[OM.OFF_B3:] = rng.normal(0, 0.1, OM.NO)
    return w


def test_mlp_kernels_match_cpu(ctx):
    """Forward outputs and parameter gradients of the GPU network kernels
    against the CPU restatement (BF16 forward, FP32 accumulation)."""
    w = _random_weights(1)
    bem.learned_set_weights(w, ctx=ctx)
    assert np.array_equal(bem.learned_get_weights(ctx=ctx), w)
    rng = np.random.default_rng(2)
    P = 3000
    F = rng.normal(size=(P, OM.NF)).astype(np.float32)
    dO = rng.normal(size=(P, OM.NO)).astype(np.float32)
    out, grad = bem.learned_mlp_eval(F, dO, ctx=ctx)
    o_ref, g_ref = OM.backward(w, F, dO)
    assert np.max(np.abs(out - o_ref)) <= 2e-2 * np.max(np.abs(o_ref))
    assert np.linalg.norm(out - o_ref) <= 3e-3 * np.linalg.norm(o_ref)
    for lo, hi in ((OM.OFF_W1, OM.OFF_B1), (OM.OFF_B1, OM.OFF_W2), (OM.OFF_W2, OM.OFF_B2),
                   (OM.OFF_B2, OM.OFF_W3), (OM.OFF_W3, OM.OFF_B3), (OM.OFF_B3, OM.NPARAM)):
        assert np.linalg.norm(grad[lo:hi] - g_ref[lo:hi]) <= 1e-2 * np.linalg.norm(g_ref[lo:hi]), (lo, hi)


@pytest.mark.parametrize("P", [1, 127, 128, 129, 5000])
def test_tensor_core_inference_matches_cpu(ctx, P):
    """tcgen05 inference (BF16 operands in shared memory, FP32 accumulators in
    tensor memory) against the CPU restatement and the CUDA-core forward."""
    w = _random_weights(7)
    bem.learned_set_weights(w, ctx=ctx)
    rng = np.random.default_rng(P)
    F = rng.normal(size=(P, OM.NF)).astype(np.float32)
    out = np.zeros((P, 2), dtype=np.float32)
    ctx.check(ctx.lib.bem_learned_mlp_infer(ctx.h, P, bem._ptr(F), bem._ptr(out)))
    ref = OM.forward(w, F)[3]
    cuda_core = bem.learned_mlp_eval(F, ctx=ctx)
    scale = max(np.max(np.abs(ref)), 1e-6)
    assert np.max(np.abs(out - ref)) <= 2e-2 * scale
    assert np.linalg.norm(out - ref) <= 3e-3 * np.linalg.norm(ref)
    # both GPU forwards round activations to BF16 with different FP32
    # summation orders: each is within 3e-3 of the restatement, so within 6e-3
    # of each other; a wrong tile row would differ by O(1)
    assert np.linalg.norm(out - cuda_core) <= 6e-3 * np.linalg.norm(cuda_core)
    assert np.max(np.abs(out - cuda_core)) <= 2e-2 * scale


def _run(ctx, inp, precond):
    a = bem.Analysis(ctx)
    a.set_input(inp)
    a.run(form="mixed", precond=precond, check_vs_lu=True)
    return a


def test_block_jacobi(ctx, workdir):
    inp = workloads.perturbed_sphere_input(workdir, 11, 900, [3.0, 6.0], tol=1e-6)
    r0 = _run(ctx, inp, None).reports
    r1 = _run(ctx, inp, "block_jacobi").reports
    for a, b in zip(r0, r1):
        assert a["flag"] == 1 and b["flag"] == 1 and b["precond"] == 1
        assert 0 <= b["rel_err_vs_lu"] < 1e-6
        assert b["iterations"] <= a["iterations"]


def test_learned_preconditioner(ctx, workdir):
    """Train on BEM operators of perturbed spheres, evaluate on a held-out body:
    the network lowers the probe loss below block-Jacobi's (its untrained
    value), the solves stay within 1e-6 of FP64 LU, and the iteration count is
    reported against block-Jacobi and no preconditioner."""
    train = [bem.PreData.from_dict(workloads.perturbed_sphere_input(workdir, s, t, [2.0, 5.0, 8.0]), ctx=ctx)
             for s, t in ((21, 600), (22, 800), (23, 700))]
    # a fresh network: random hidden layers, W3 = b3 = 0 so the correction
    # starts at zero (= block-Jacobi)
    w0 = _random_weights(3)
    w0[OM.OFF_W3:] = 0.0
    bem.learned_set_weights(w0, ctx=ctx)
    losses = bem.learned_train(train, steps=180, nprobe=8, lr=2e-3, seed=5, ctx=ctx)
    assert np.all(np.isfinite(losses))
    first, last = np.mean(losses[:9]), np.mean(losses[-9:])
    assert last < first
    held = workloads.perturbed_sphere_input(workdir, 99, 1000, [4.0, 7.0], tol=1e-6)
    rn = _run(ctx, held, None).reports
    rb = _run(ctx, held, "block_jacobi").reports
    rl = _run(ctx, held, "learned").reports
    for a, b, c in zip(rn, rb, rl):
        assert c["flag"] == 1 and c["precond"] == 2
        assert 0 <= c["rel_err_vs_lu"] < 1e-6
        assert c["iterations"] <= a["iterations"]
    print("iterations none/bj/learned:", [r["iterations"] for r in rn], [r["iterations"] for r in rb],
          [r["iterations"] for r in rl], "loss %.4g -> %.4g" % (first, last))

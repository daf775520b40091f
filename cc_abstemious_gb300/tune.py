"""Offline sweep of the tunable launch parameters (run on the GPU).

    python -m cc_abstemious_gb300.tune [--out cc_abstemious_gb300/tuning.json]

For every tunable kernel and every representative size, each candidate value
is forced on a context (bem_ctx_set_tuning), a representative workload of that
size runs twice with the library's per-stage CUDA-event timing, and the second
run's time of the kernel's stage is kept.  The fastest candidate becomes the
table entry; the entry also records every candidate's time and the built-in
default's, so the gain of the table is on file.  A context reads the table
(tuning.json beside the library) at creation.

  lu_gemm_trail  (sb_r, sb_c): tile raster of the trailing update (stage
                 lu_gemm_trail) -- mixed form with the LU preconditioner, one
                 frequency of cube-spheres of 1944 .. 40344 quads, and a batch
                 of 64 perturbed spheres; group: block steps per pass over A22
                 (4 or 8; stage lu_setup_total, the whole factorization) on the
                 spheres from 12000 quads.
  gm_apply_fp32  unroll: columns per load batch of the Krylov mat-vec (stage
                 gmres_matvec_fp32) -- the rigid sphere, 16 frequencies.
  assemble32     min_ctas: occupancy bound of the FP32 assembly (stage
                 assemble_fp32) -- the same runs.
"""
import argparse
import ctypes as C
import json
import os
import tempfile
import time

import numpy as np

from . import _lib, workloads

HERE = os.path.dirname(os.path.abspath(__file__))

RASTERS = [(65535, 1), (4, 64), (8, 32), (16, 32), (8, 16), (32, 8)]
UNROLLS = [4, 8, 16]
MINB = [2, 3, 4]


def _stage_ms(ctx, run, stage):
    ctx.set_profiling(True)
    run()
    run()
    prof = ctx.profile()
    ctx.set_profiling(False)
    return prof.get(stage, {}).get("ms")


def _set(ctx, kernel, params):
    for k, v in params.items():
        ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, kernel.encode(), k.encode(), int(v)))


def _clear(ctx, kernel, params):
    for k in params:
        ctx.check(ctx.lib.bem_ctx_set_tuning(ctx.h, kernel.encode(), k.encode(), -1))


def sweep(kernel, candidates, cases, default):
    """cases: [(n, nsys, ctx, run, stage)] -> table entries."""
    out = []
    for n, nsys, ctx, run, stage in cases:
        times = []
        for cand in candidates:
            _set(ctx, kernel, cand)
            ms = _stage_ms(ctx, run, stage)
            _clear(ctx, kernel, cand)
            times.append((ms, cand))
            print("  %-14s n=%-6d nsys=%-4d %-26s %8.3f ms" % (kernel, n, nsys, json.dumps(cand), ms), flush=True)
        best = min(times, key=lambda t: t[0])
        dflt = [t for t in times if t[1] == default]
        out.append({"kernel": kernel, "n": n, "nsys": nsys, "params": best[1], "ms": best[0],
                    "default": default, "default_ms": dflt[0][0] if dflt else None,
                    "candidates": [{"params": c, "ms": t} for t, c in times]})
    return out


def main():
    import cc_abstemious_gb300 as bem
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "tuning.json"))
    ap.add_argument("--sizes", default="18,32,58,82", help="cube-sphere subdivisions for the LU sweep")
    args = ap.parse_args()
    os.environ["BEM_TUNING_FILE"] = "none"  # time the candidates, not an earlier table
    ctx = bem.Context(0)
    wd = tempfile.mkdtemp(prefix="bem_tune_")
    entries = []
    t0 = time.time()

    # the LU trailing update on single operators and a batch
    cases = []
    for m in [int(x) for x in args.sizes.split(",")]:
        inp = workloads.rigid_sphere_bm(wd, m=m, nfreq=1, ka_lo=6.0, ka_hi=6.0)
        pd = bem.PreData.from_dict(inp, ctx=ctx)
        nf = len(pd.frequencies)
        sc = np.zeros((nf, pd.nfp), dtype=np.complex128)

        def run(pd=pd, sc=sc, nf=nf):
            ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_MIXED, bem.PRECOND_LU, bem._ptr(sc), bem._ptr(sc),
                                      None, 0))
        cases.append((pd.n, 1, ctx, run, "lu_gemm_trail"))
    bodies = workloads.perturbed_spheres(wd, count=64, seed=3, nfreq=1, tol=1e-8)
    bpds = [bem.PreData.from_dict(d, ctx=ctx) for d in bodies]
    cases.append((int(max(p.n for p in bpds)), 64, ctx, lambda: bem.run_batch(bpds, precond="lu", ctx=ctx),
                  "lu_gemm_trail"))
    entries += sweep("lu_gemm_trail", [{"sb_r": r, "sb_c": c} for r, c in RASTERS], cases,
                     {"sb_r": 8, "sb_c": 32})
    big = [(n, ns, cx, run, "lu_setup_total") for n, ns, cx, run, _ in cases if n >= 12000 and ns == 1]
    entries += sweep("lu_gemm_trail", [{"group": g} for g in (4, 8)], big, {"group": 8})

    # the Krylov mat-vec and the FP32 assembly on the rigid sphere
    cases_mv, cases_as = [], []
    for m in (16, 32):
        inp = workloads.rigid_sphere_bm(wd, m=m, nfreq=16)
        pd = bem.PreData.from_dict(inp, ctx=ctx)
        sc = np.zeros((16, pd.nfp), dtype=np.complex128)

        def run(pd=pd, sc=sc):
            ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_MIXED, 0, bem._ptr(sc), bem._ptr(sc), None, 0))
        cases_mv.append((pd.n, 16, ctx, run, "gmres_matvec_fp32"))
        cases_as.append((pd.n, 16, ctx, run, "assemble_fp32"))
    entries += sweep("gm_apply_fp32", [{"unroll": u} for u in UNROLLS], cases_mv, {"unroll": 8})
    entries += sweep("assemble32", [{"min_ctas": b} for b in MINB], cases_as, {"min_ctas": 3})

    import torch
    table = {"version": 1, "device": torch.cuda.get_device_name(0), "seconds": time.time() - t0,
             "how": "python -m cc_abstemious_gb300.tune: every candidate timed by the library's per-stage CUDA "
                    "events (second of two runs); the fastest is the entry",
             "entries": entries}
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    print("wrote", args.out, "in %.0f s" % table["seconds"])


if __name__ == "__main__":
    main()

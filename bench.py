#!/usr/bin/env python
"""Benchmark: solves/s of the cc_abstemious hot path on one GB300.

Workload (rigid_sphere_bm): rigid sphere r = 1 m meshed as a cube-sphere of
6144 bilinear quads, exterior Burton-Miller, unit plane wave along +z, 16
frequencies with ka evenly spaced 1..10, GMRES restart 50 (max_iterations 2500)
tolerance 1e-8, 100 field points on r = 5 m.  Synthetic, seeded geometry (no
dataset).  One step = one pass of the whole hot path over the 16 frequencies:
assembly, surface solve and field evaluation -> 16 solves.

Arms:
  default        the batched mixed-precision form (FP32 operators with float-float
                 phase, FP64 GMRES), problem resident on the device; the plain FP64
                 form is timed beside it ("plain_fp64"), and the error of every
                 reported frequency against an FP64 LU of the same operator is
                 measured after the timed region.
  --impl reference  the CPU restatement of the reference algorithm (oracle/),
                 host cores only, a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s at ≤1e-6 rel err vs FP64 LU: learned+mixed vs plain FP64, 1 GB300"
UNIT = "solves/s"
WORKLOAD = "rigid_sphere_bm"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--lu-check", type=int, default=4,
                    help="frequencies checked against an FP64 LU (evenly spread; 0 = all)")
    ap.add_argument("--cpu-sample", type=int, default=2,
                    help="frequencies solved by the CPU baseline per step (evenly spread: 2 = lowest and highest ka)")
    ap.add_argument("--precond", default="none", choices=["none", "block_jacobi", "learned", "lu"])
    ap.add_argument("--mesh-m", type=int, default=32, help="cube-sphere subdivisions (6 m^2 quads)")
    ap.add_argument("--nfreq", type=int, default=16)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--profile-only", action="store_true", help="one mixed run (for ncu launch lists)")
    ap.add_argument("--workload", default=WORKLOAD,
                    choices=[WORKLOAD, "perturbed_spheres", "held_out_learned", "ellipsoid_bm"],
                    help="rigid_sphere_bm (the metric's configuration, default); perturbed_spheres (bodies of "
                         "500-5000 triangles x 8 frequencies in one batch); held_out_learned (learned vs "
                         "block-Jacobi on a held-out 20000-triangle body); ellipsoid_bm (40960 triangles, "
                         "two right-hand sides, 8 frequencies up to ka 20)")
    ap.add_argument("--bodies", type=int, default=256, help="perturbed_spheres: number of bodies")
    ap.add_argument("--train-bodies", type=int, default=16, help="held_out_learned: training bodies")
    ap.add_argument("--train-steps", type=int, default=400, help="held_out_learned: training steps")
    ap.add_argument("--held-out-tri", type=int, default=20000, help="held_out_learned: triangles")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(ms, world, device):
    """The slowest rank's time: every replica's step must be over before the
    whole job's is."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(solves_per_rank, ms_max, world):
    """Solves per second of the whole job: every rank solved its own copy of
    the workload (replicas, weak scaling) within the slowest rank's time."""
    return world * solves_per_rank * 1000.0 / ms_max


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def ncu_traffic_ratio():
    """DRAM traffic / algorithmic bytes of the batched FP32 mat-vec, from the
    committed ncu summary (profiles/); traffic scales with the matrices streamed."""
    p = os.path.join(ROOT, "profiles", "gm_apply_fp32_rigid_sphere_bm.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_over_algorithmic:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def tf32_peak():
    """cuBLAS TF32 GEMM throughput measured in this run (8192^3, best of 5,
    CUDA events): the denominator for the TF32 tensor-core LU update, since the
    measured peaks file covers HBM and BF16 only."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    n = 8192
    a = torch.randn(n, n, device="cuda")
    b = torch.randn(n, n, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for i in range(7):
        e0.record()
        c = a @ b
        e1.record()
        e1.synchronize()
        if i >= 2:
            best = min(best, e0.elapsed_time(e1))
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b, c
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def lu_traffic_ratio():
    """DRAM traffic / algorithmic A22 bytes of one K = 1024 trailing update, from
    the committed ncu summary (profiles/)."""
    p = os.path.join(ROOT, "profiles", "lu_gemm_tf32_group_rigid_sphere.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_over_algorithmic:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def lu_roofline(prof, sizes, what):
    """Roofline entry of the LU preconditioner's trailing update (the dominant
    kernel of the LU forms): TF32 flop rate of the lu_gemm launches (event-timed
    by the library's profiling pass; 8 n^3 / 3 complex flop per factored
    operator) against cuBLAS TF32 measured here.  Block steps run in groups of
    four: one K = 1024 launch per group reads and writes the rest of the
    trailing block once, so its algorithmic bytes are 16 B (FP32 complex, read
    + write) per entry of that block (reported per operator: a launch covers
    every operator of a frequency chunk)."""
    lu = prof.get("lu_gemm_tf32", {})
    achieved = lu["bytes"] / (lu["ms"] * 1e-3) / 1e12 if lu.get("ms") else None
    peak = tf32_peak()
    lb, group = 128, 4
    tot, cnt = 0.0, 0
    for n in sizes:
        nblk = (n + lb - 1) // lb
        for k in range(0, nblk, group):
            m1 = n - (k + group) * lb
            if m1 > 0:
                tot += 16.0 * m1 * m1
                cnt += 1
    alg = tot / cnt if cnt else None
    ratio = lu_traffic_ratio()
    return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if achieved else None,
            "traffic": ratio * alg if (ratio and alg) else None,
            "kernel": "lu_gemm_kernel<TRAIL> (TF32 tcgen05 trailing update of the LU preconditioner, " + what + ")",
            "algorithmic_bytes_per_operator_launch": alg,
            "peak_kind": "measured in this run (cuBLAS TF32 GEMM 8192^3, burst)",
            "traffic_note": "ncu dram read+write / algorithmic A22 bytes of one K = 1024 launch "
                            "(profiles/lu_gemm_tf32_group_rigid_sphere.md), times the mean algorithmic bytes "
                            "of this workload's K = 1024 launches, per operator"}


def cpu_reference(inp, nfreq_sample, threads):
    """The oracle (C restatement of the reference algorithm) on `nfreq_sample`
    frequencies of the workload; returns (solves/s, seconds, sample text)."""
    from oracle import oracle as O
    import numpy as np
    freqs = inp["frequency"]["List"]["values"]
    idx = np.linspace(0, len(freqs) - 1, nfreq_sample).round().astype(int)
    sample = dict(inp, frequency={"List": {"values": [freqs[i] for i in idx]}})
    P = O.Problem(sample)
    t0 = time.perf_counter()
    P.run(nthreads=threads)
    dt = time.perf_counter() - t0
    return nfreq_sample / dt, dt, "%d of the %d frequencies (%s Hz), N=%d" % (
        nfreq_sample, len(freqs), ",".join("%.1f" % freqs[i] for i in idx), P.n)


def run_reference_arm(args, inp):
    rank, world, local = dist_env()
    if rank != 0:
        return
    threads = max((os.cpu_count() or 2) // 2, 2)  # preprocess.rs:12-17
    vals = []
    for _ in range(args.warmup):
        cpu_reference(inp, args.cpu_sample, threads)
    t_total = 0.0
    for _ in range(max(args.steps, 1)):
        v, dt, sample = cpu_reference(inp, args.cpu_sample, threads)
        vals.append(v)
        t_total += dt
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 complex",
            "data": "synthetic (seeded cube-sphere mesh)",
            "config": {"workload": WORKLOAD, "n_unknowns": 6 * args.mesh_m ** 2, "frequencies": args.nfreq,
                       "parallelism": "replicas only"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample + " per step; oracle/ C restatement of the reference "
                                                "(reference Rust toolchain absent)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "perturbed_spheres":
        return bench_perturbed_spheres(args)
    if args.workload == "held_out_learned":
        return bench_held_out_learned(args)
    if args.workload == "ellipsoid_bm":
        return bench_ellipsoid(args)
    rank, world, local = dist_env()
    from cc_abstemious_gb300 import workloads
    workdir = tempfile.mkdtemp(prefix="bem_bench_")
    inp = workloads.rigid_sphere_bm(workdir, m=args.mesh_m, nfreq=args.nfreq)
    if args.impl == "reference":
        run_reference_arm(args, inp)
        return

    import numpy as np
    import torch
    import cc_abstemious_gb300 as bem
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    text = json.dumps(inp)
    ctx = bem.Context(local)
    pd = bem.PreData.from_json(text, ctx=ctx)
    nf = len(pd.frequencies)
    stream = torch.cuda.ExternalStream(ctx.stream)
    precond = {"none": 0, "block_jacobi": 1, "learned": 2, "lu": 3}[args.precond]
    sc = np.zeros((nf, pd.nfp), dtype=np.complex128)
    inc = np.zeros((nf, pd.nfp), dtype=np.complex128)
    reps = (bem.SolveReport * nf)()

    def run_mixed(check=0):
        ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_MIXED, precond, bem._ptr(sc), bem._ptr(inc), reps, check))

    if args.profile_only:
        run_mixed()
        torch.cuda.synchronize()
        return

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        run_mixed()
    iters = [r.iterations for r in reps]

    # ---- timed region: device-resident problem, CUDA events on the library stream
    launches0 = ctx.kernel_launches
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)  # sampler running before the timed region starts
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        run_mixed()
    e1.record(stream)
    e1.synchronize()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    gpu_launches = ctx.kernel_launches - launches0
    ms_all = max_over_ranks(ms, world, "cuda")
    value = whole_job_rate(nf, ms_all, world)

    # ---- end to end through the public API: JSON text + mesh file on the host ->
    # preprocessing on the device -> every frequency -> results in host memory
    mesh_bytes = os.path.getsize(inp["mesh_file"])
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        a = bem.Analysis(ctx)
        a.input_from_string(text)
        a.run(form="mixed", precond=None if args.precond == "none" else args.precond)
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_ms = max_over_ranks(e2e_s * 1000.0, world, "cuda")
    e2e_value = whole_job_rate(nf, e2e_ms, world)
    info = pd.info
    h2d = 8 * 3 * info["mesh_nodes"] + 8 * 5 * pd.n + 8 * 3 * pd.nfp  # nodes, element table, field points
    d2h = 16 * 2 * nf * pd.nfp + 16 * 2 * nf * pd.n + 8 * 9 * pd.n  # results, surface solution, collocation

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        return

    # ---- plain FP64 drop-in form on the same workload (one step)
    plain = None
    if not args.no_plain:
        reps_p = (bem.SolveReport * nf)()
        ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(sc), bem._ptr(inc), reps_p, 0))
        ep0, ep1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ep0.record(stream)
        ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(sc), bem._ptr(inc), reps_p, 0))
        ep1.record(stream)
        ep1.synchronize()
        pms = ep0.elapsed_time(ep1)
        plain = {"value": nf * 1000.0 / pms, "unit": UNIT, "ms_per_step": pms,
                 "iterations": [r.iterations for r in reps_p]}
        sc_plain = sc.copy()

    # ---- accuracy: mixed vs an FP64 LU of the same operator, sampled frequencies
    run_mixed(check=0)
    sc_mixed = sc.copy()
    errs = {}
    idx = list(range(nf)) if args.lu_check == 0 else sorted(set(
        int(round(x)) for x in np.linspace(0, nf - 1, min(args.lu_check, nf))))
    for i in idx:
        one = dict(inp, frequency={"List": {"values": [inp["frequency"]["List"]["values"][i]]}})
        p1 = bem.PreData.from_json(json.dumps(one), ctx=ctx)
        r1 = (bem.SolveReport * 1)()
        s1 = np.zeros((1, pd.nfp), dtype=np.complex128)
        i1 = np.zeros((1, pd.nfp), dtype=np.complex128)
        ctx.check(ctx.lib.bem_run(ctx.h, p1.h, bem.FORM_MIXED, precond, bem._ptr(s1), bem._ptr(i1), r1, 1))
        errs["%.3f" % (1.0 + 9.0 * i / max(nf - 1, 1))] = r1[0].rel_err_vs_lu
        del p1
    field_err_vs_plain = None
    if plain is not None:
        field_err_vs_plain = float(np.max(np.abs(sc_mixed - sc_plain)) / np.max(np.abs(sc_plain)))

    # ---- per-kernel timing pass (CUDA events around every Krylov mat-vec)
    ctx.set_profiling(True)
    run_mixed()
    prof = ctx.profile()
    ctx.set_profiling(False)
    hbm_peak, peak_kind = measured_peaks()
    mv = prof.get("gmres_matvec_fp32", {})
    achieved = mv["bytes"] / (mv["ms"] * 1e-3) / 1e9 if mv.get("ms") else None
    ratio = ncu_traffic_ratio()
    alg_per_launch = mv["bytes"] / max(mv["launches"], 1) if mv else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak if achieved else None,
                "traffic": ratio * alg_per_launch if (ratio and alg_per_launch) else None,
                "kernel": "gm_apply_kernel<float2, 0> (batched FP32-operator Krylov mat-vec)",
                "algorithmic_bytes_per_launch": alg_per_launch,
                "peak_kind": peak_kind + " (burst copy)",
                "traffic_note": "ncu dram read+write / algorithmic bytes from profiles/"
                                "gm_apply_fp32_rigid_sphere_bm.md (small case), scaled to this launch"}

    # ---- CPU baseline: the oracle on a bounded sample, host cores of this machine
    threads = max((os.cpu_count() or 2) // 2, 2)
    cv, cdt, sample = cpu_reference(inp, args.cpu_sample, threads)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_all, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 operator / fp64 vectors (complex)",
        "data": "synthetic (cube-sphere mesh, no dataset)",
        "config": {"workload": WORKLOAD, "n_unknowns": pd.n, "frequencies": nf, "ka": [1.0, 10.0],
                   "solver": "GMRES restart 50 tol 1e-8", "field_points": pd.nfp,
                   "form": "batched mixed (FP32 assembly + FP64 GMRES)",
                   "precond": args.precond, "l2": "operators 8 B x N^2 x 16 = %.1f GB > L2 (no flush needed)"
                   % (8.0 * pd.n * pd.n * nf / 1e9), "parallelism": "replicas only"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "mesh_file_bytes": mesh_bytes, "note": "JSON text + VTK file on host -> results on host"},
        "gpu_launches": gpu_launches,
        "roofline": roofline,
        "cpu_baseline": {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample + "; oracle/ C restatement, reference thread count max(nproc/2,2)"},
        "clocks": clk,
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
        "rel_err_vs_fp64_lu": errs,
        "max_rel_err_vs_fp64_lu": max(errs.values()) if errs else None,
        "field_rel_diff_vs_plain": field_err_vs_plain,
        "gmres_iterations": iters,
        "stages_ms": {k: v["ms"] for k, v in prof.items()},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# Further workloads (one JSON line each, same keys as the default line).

def _timed_region(args, device, fn, stream):
    """W warm-up calls, then K calls between CUDA events on the library stream,
    clocks sampled meanwhile; returns (ms per call, clocks)."""
    import torch
    for _ in range(max(args.warmup, 3)):
        fn()
    clocks = Clocks(device)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    return e0.elapsed_time(e1) / args.steps, clk


def _roofline_from_profile(prof, what):
    hbm_peak, peak_kind = measured_peaks()
    mv = prof.get("gmres_matvec_fp32", {})
    achieved = mv["bytes"] / (mv["ms"] * 1e-3) / 1e9 if mv.get("ms") else None
    ratio = ncu_traffic_ratio()
    alg = mv["bytes"] / max(mv["launches"], 1) if mv else None
    return {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak if achieved else None,
            "traffic": ratio * alg if (ratio and alg) else None,
            "kernel": "gm_apply_kernel<float2, 0> (" + what + ")", "algorithmic_bytes_per_launch": alg,
            "peak_kind": peak_kind + " (burst copy)",
            "traffic_note": "ncu dram read+write / algorithmic bytes of the same kernel on the rigid-sphere "
                            "case (profiles/gm_apply_fp32_rigid_sphere_bm.md), scaled to this launch"}


def bench_perturbed_spheres(args):
    """Bodies r = 1 + sum a_lm Y_lm (l <= 4), 500-5000 triangles each, impedance
    Z = rho c (1 + 0.2 i), Burton-Miller, 8 frequencies ka 0.5..8 each: all
    bodies and frequencies in one batch (bem_run_batch).  GMRES tolerance 1e-8
    on the backward error, so the forward error stays below 1e-6."""
    import numpy as np
    import torch
    import cc_abstemious_gb300 as bem
    from cc_abstemious_gb300 import workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    workdir = tempfile.mkdtemp(prefix="bem_bench_ps_")
    inps = workloads.perturbed_spheres(workdir, count=args.bodies, seed=0, nfreq=8, tol=1e-8)
    if args.impl == "reference":
        return _reference_arm_generic(args, inps[len(inps) // 2], "perturbed_spheres",
                                      {"bodies": len(inps), "frequencies_per_body": 8})
    ctx = bem.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    texts = [json.dumps(d) for d in inps]
    pds = [bem.PreData.from_json(t, ctx=ctx) for t in texts]
    ns = [pd.n for pd in pds]
    nsys = sum(len(pd.frequencies) for pd in pds)
    pc = None if args.precond == "none" else args.precond
    last = {}

    def step():
        last["out"] = bem.run_batch(pds, precond=pc, ctx=ctx)

    launches0 = ctx.kernel_launches
    ms, clk = _timed_region(args, local, step, stream)
    gpu_launches = (ctx.kernel_launches - launches0) * args.steps // (args.steps + max(args.warmup, 3))
    value = world * nsys * 1000.0 / ms
    iters = [r["iterations"] for _, reps in last["out"] for r in reps]

    # end to end: JSON text + mesh files on the host -> results on the host
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        p2 = [bem.PreData.from_json(t, ctx=ctx) for t in texts]
        bem.run_batch(p2, precond=pc, ctx=ctx)
        del p2
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    nfp = pds[0].nfp
    h2d = sum(8 * 3 * pd.info["mesh_nodes"] + 8 * 5 * pd.n + 8 * 3 * pd.nfp for pd in pds)
    d2h = sum(16 * 2 * len(pd.frequencies) * pd.nfp for pd in pds)

    # plain FP64 drop-in form, body by body (one pass)
    plain = None
    if not args.no_plain:
        sc = np.zeros((8, nfp), dtype=np.complex128)
        inc = np.zeros((8, nfp), dtype=np.complex128)
        reps = (bem.SolveReport * 8)()
        ep0, ep1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ep0.record(stream)
        pit = []
        for pd in pds:
            ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(sc), bem._ptr(inc), reps, 0))
            pit += [reps[i].iterations for i in range(len(pd.frequencies))]
        ep1.record(stream)
        ep1.synchronize()
        pms = ep0.elapsed_time(ep1)
        plain = {"value": nsys * 1000.0 / pms, "unit": UNIT, "ms_per_step": pms,
                 "iterations_mean": float(np.mean(pit)), "iterations_max": int(max(pit))}

    # error against FP64 LU: the smallest, a middle and the largest body, all
    # their frequencies (each system's GMRES is independent of the others)
    order = np.argsort(ns)
    pick = sorted({int(order[0]), int(order[len(order) // 2]), int(order[-1])})
    chk = bem.run_batch([pds[i] for i in pick], precond=pc, check_vs_lu=True, ctx=ctx)
    errs = {"body%d_N%d" % (i, ns[i]): max(r["rel_err_vs_lu"] for r in reps) for i, (_, reps) in zip(pick, chk)}

    ctx.set_profiling(True)
    bem.run_batch(pds, precond=pc, ctx=ctx)
    prof = ctx.profile()
    ctx.set_profiling(False)
    if pc == "lu":
        roofline = lu_roofline(prof, list(ns), "ragged batch over all bodies and frequencies")
    else:
        roofline = _roofline_from_profile(prof, "ragged batch over all bodies and frequencies")

    threads = max((os.cpu_count() or 2) // 2, 2)
    mid = int(order[len(order) // 2])
    cv, cdt, sample = cpu_reference(inps[mid], 1, threads)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 operator / fp64 vectors (complex)" + ("; tf32 LU preconditioner" if pc == "lu" else ""),
        "data": "synthetic (seeded harmonic-perturbed spheres, no dataset)",
        "config": {"workload": "perturbed_spheres", "bodies": len(pds), "frequencies_per_body": 8,
                   "systems": nsys, "n_min": int(min(ns)), "n_max": int(max(ns)), "n_mean": float(np.mean(ns)),
                   "ka": [0.5, 8.0], "bc": "impedance rho c (1 + 0.2i)", "solver": "GMRES tol 1e-8",
                   "form": "one multi-body assembly launch + one ragged batched GMRES",
                   "precond": args.precond,
                   "l2": "operators %.1f GB > L2 (no flush needed)" % (8e-9 * sum(
                       (-(-pd.n // 64) * 64) * pd.n * len(pd.frequencies) for pd in pds)),
                   "parallelism": "replicas only"},
        "e2e": {"value": world * nsys * 1000.0 / e2e_ms, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "note": "JSON text + VTK files on host -> results on host"},
        "gpu_launches": gpu_launches, "roofline": roofline,
        "cpu_baseline": {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample + "; the median-size body; oracle/ C restatement"},
        "clocks": clk, "plain_fp64": plain,
        "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
        "rel_err_vs_fp64_lu": errs, "max_rel_err_vs_fp64_lu": max(errs.values()),
        "gmres_iterations_mean": float(np.mean(iters)), "gmres_iterations_max": int(max(iters)),
        "stages_ms": {k: v["ms"] for k, v in prof.items()},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_held_out_learned(args):
    """Learned preconditioner on a held-out body: the network is trained on the
    GPU on operators of perturbed spheres drawn like the batch workload, then a
    held-out sphere of the same distribution (20000 triangles, ka 4..16 at 12
    frequencies, GMRES tolerance 1e-6) is solved with no preconditioner,
    block-Jacobi and the learned correction."""
    import numpy as np
    import torch
    import cc_abstemious_gb300 as bem
    from cc_abstemious_gb300 import workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    workdir = tempfile.mkdtemp(prefix="bem_bench_lh_")
    kas = np.linspace(4.0, 16.0, 12)
    # GMRES stops on the backward error; 1e-8 keeps the forward error against
    # FP64 LU below 1e-6 (at 1e-6 the forward error reaches ~1.3e-6 here)
    held = workloads.perturbed_sphere_input(workdir, 777777, args.held_out_tri, kas, tol=1e-8)
    if args.impl == "reference":
        return _reference_arm_generic(args, held, "held_out_learned", {"n_triangles": args.held_out_tri})
    ctx = bem.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    train = workloads.perturbed_spheres(workdir, count=args.train_bodies, seed=1, nfreq=8, tri_lo=500,
                                        tri_hi=3000)
    tpds = [bem.PreData.from_dict(d, ctx=ctx) for d in train]
    t0 = time.perf_counter()
    losses = bem.learned_train(tpds, steps=args.train_steps, nprobe=8, lr=2e-3, seed=5, ctx=ctx)
    train_s = time.perf_counter() - t0
    del tpds
    pd = bem.PreData.from_dict(held, ctx=ctx)
    nf = len(pd.frequencies)
    sc = np.zeros((nf, pd.nfp), dtype=np.complex128)
    inc = np.zeros((nf, pd.nfp), dtype=np.complex128)
    results = {}
    forms = {"none": (bem.FORM_MIXED, 0), "block_jacobi": (bem.FORM_MIXED, 1), "learned": (bem.FORM_MIXED, 2),
             "lu": (bem.FORM_MIXED, 3), "lu_refined": (bem.FORM_REFINED, 3)}
    for name, (form, code) in forms.items():
        reps = (bem.SolveReport * nf)()

        def step():
            ctx.check(ctx.lib.bem_run(ctx.h, pd.h, form, code, bem._ptr(sc), bem._ptr(inc), reps, 0))

        launches0 = ctx.kernel_launches
        ms, clk = _timed_region(args, local, step, stream)
        launches = (ctx.kernel_launches - launches0) * args.steps // (args.steps + max(args.warmup, 3))
        results[name] = {"value": nf * 1000.0 / ms, "ms_per_step": ms, "clocks": clk, "gpu_launches": launches,
                         "iterations": [reps[i].iterations for i in range(nf)],
                         "converged": all(reps[i].flag == 1 for i in range(nf)),
                         "precond_used": [reps[i].precond for i in range(nf)]}
    # the headline form: the fastest whose every system converged and whose
    # error against FP64 LU (lowest and highest ka) is within 1e-6
    def lu_errors(name):
        form, code = forms[name]
        out = {}
        for i in (0, nf - 1):
            one = dict(held, frequency={"List": {"values": [held["frequency"]["List"]["values"][i]]}})
            p1 = bem.PreData.from_dict(one, ctx=ctx)
            r1 = (bem.SolveReport * 1)()
            s1 = np.zeros((1, pd.nfp), dtype=np.complex128)
            ctx.check(ctx.lib.bem_run(ctx.h, p1.h, form, code, bem._ptr(s1), bem._ptr(s1), r1, 1))
            out["ka%.2f" % kas[i]] = r1[0].rel_err_vs_lu
            del p1
        return out

    ok = sorted([k for k in results if results[k]["converged"]] or list(results),
                key=lambda k: -results[k]["value"])
    best, errs = ok[0], {}
    for cand in ok:
        e = lu_errors(cand)
        results[cand]["rel_err_vs_fp64_lu"] = e
        best, errs = cand, e
        if max(e.values()) <= 1e-6:
            break
    form_best, code_best = forms[best]
    plain = None
    if not args.no_plain:
        reps = (bem.SolveReport * nf)()
        ep0, ep1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ep0.record(stream)
        ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(sc), bem._ptr(inc), reps, 0))
        ep1.record(stream)
        ep1.synchronize()
        pms = ep0.elapsed_time(ep1)
        plain = {"value": nf * 1000.0 / pms, "unit": UNIT, "ms_per_step": pms,
                 "iterations": [reps[i].iterations for i in range(nf)]}
    ctx.set_profiling(True)
    ctx.check(ctx.lib.bem_run(ctx.h, pd.h, form_best, code_best, bem._ptr(sc), bem._ptr(inc),
                              (bem.SolveReport * nf)(), 0))
    prof = ctx.profile()
    ctx.set_profiling(False)
    value = results[best]["value"]
    # end to end through the public API (JSON text + mesh file on the host ->
    # results on the host), the headline form
    text = json.dumps(held)
    fname = {bem.FORM_MIXED: "mixed", bem.FORM_REFINED: "refined"}[form_best]
    pname = {0: None, 1: "block_jacobi", 2: "learned", 3: "lu"}[code_best]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        a = bem.Analysis(ctx)
        a.input_from_string(text)
        a.run(form=fname, precond=pname)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    if code_best == 3:
        roofline = lu_roofline(prof, [pd.n], "12 frequencies of the held-out body, " + best)
    else:
        roofline = _roofline_from_profile(prof, "12 frequencies of the held-out body, " + best)
    # CPU baseline: the oracle on one frequency of a smaller body of the same
    # distribution (its dense FP64 LU of 20000 unknowns is not a bounded sample)
    threads = max((os.cpu_count() or 2) // 2, 2)
    small = workloads.perturbed_sphere_input(workdir, 777777, 2000, kas, tol=1e-8)
    cv, cdt, sample = cpu_reference(small, 1, threads)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": results[best]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("fp64 operator / tf32 LU preconditioner (complex)" if form_best == bem.FORM_REFINED else
                  "fp32 operator / fp64 vectors (complex)" + ("; tf32 LU preconditioner" if code_best == 3 else
                                                             "; bf16 network" if code_best == 2 else "")),
        "data": "synthetic (seeded harmonic-perturbed spheres, no dataset)",
        "config": {"workload": "held_out_learned", "n_unknowns": pd.n, "frequencies": nf, "ka": [4.0, 16.0],
                   "solver": "GMRES tol 1e-8 (backward error; 1e-6 leaves ~1.3e-6 forward error)",
                   "precond": best,
                   "precond_note": "value = fastest form with every system converged and its error "
                                   "against FP64 LU within 1e-6; every candidate is listed under by_precond "
                                   "(lu_refined: FP64 operator, TF32 LU preconditioner)",
                   "training": {"bodies": len(train), "steps": args.train_steps, "seconds": train_s,
                                "loss_first": float(np.mean(losses[:10])), "loss_last": float(np.mean(losses[-10:]))},
                   "parallelism": "replicas only"},
        "clocks": results[best]["clocks"], "by_precond": results, "plain_fp64": plain,
        "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
        "rel_err_vs_fp64_lu": errs, "max_rel_err_vs_fp64_lu": max(errs.values()),
        "e2e": {"value": world * nf * 1000.0 / e2e_ms, "unit": UNIT,
                "h2d_bytes_per_step": 8 * 3 * pd.info["mesh_nodes"] + 8 * 5 * pd.n + 8 * 3 * pd.nfp,
                "d2h_bytes_per_step": 16 * 2 * nf * pd.nfp, "note": "JSON text + VTK file on host -> results on host"},
        "gpu_launches": results[best]["gpu_launches"],
        "roofline": roofline,
        "cpu_baseline": {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample + "; a 2000-triangle body of the same distribution and seed"},
        "stages_ms": {k: v["ms"] for k, v in prof.items()},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_ellipsoid(args):
    """Ellipsoid (2, 1, 0.5) m with 40960 triangles, Burton-Miller, a plane wave
    along a seeded direction and a point source at (0, 0, 3), 8 frequencies with
    ka (a = 2) 2.5..20: 16 solves per step.  The input asks for the H-matrix
    solver at tolerance 1e-6; the forms measured here solve the dense operators
    (8 x 40960^2) with the TF32 LU preconditioner, at backward error 1e-8: the
    mixed form (FP32 operators) and the refined form (FP64 operators) are both
    timed and the headline is the faster one whose every solve is within 1e-6.
    The error reference is the same FP64 operator solved to backward error
    1e-12 (a dense FP64 LU of 40960 unknowns per frequency is too slow for a
    benchmark; both forms are checked against FP64 LU at smaller sizes in the
    tests)."""
    import numpy as np
    import torch
    import cc_abstemious_gb300 as bem
    from cc_abstemious_gb300 import workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    workdir = tempfile.mkdtemp(prefix="bem_bench_el_")
    pw, ps = workloads.ellipsoid_bm(workdir)
    if args.impl == "reference":
        coarse = workloads.ellipsoid_bm(workdir, n_lon=64, n_bands=21)[0]
        return _reference_arm_generic(args, coarse, "ellipsoid_bm", {"n_triangles": 40960,
                                                                     "sample_triangles": 2560})

    def with_tol(inp, tol):
        d = json.loads(json.dumps(inp))
        d["solver"]["Hierarchical"]["tolerance"] = tol
        return d

    ctx = bem.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    # both waves in one input (extension key additional_incident_waves): each
    # frequency's operator is assembled and factored once for the two
    both = with_tol(pw, 1e-8)
    both["additional_incident_waves"] = [ps["incident_wave"]]
    texts = [json.dumps(both)]
    pds = [bem.PreData.from_json(t, ctx=ctx) for t in texts]
    nf = len(pds[0].frequencies)
    nfp = pds[0].nfp
    R = 2
    nsolve = nf * R
    out2 = np.zeros((R * nf, nfp), dtype=np.complex128)
    inc = np.zeros((R * nf, nfp), dtype=np.complex128)
    reps2 = (bem.SolveReport * (R * nf))()

    def step(form=bem.FORM_REFINED):
        ctx.check(ctx.lib.bem_run(ctx.h, pds[0].h, form, 3, bem._ptr(out2), bem._ptr(inc), reps2, 0))

    outs = [out2[:nf], out2[nf:]]
    reps = [[reps2[i] for i in range(nf)], [reps2[nf + i] for i in range(nf)]]

    # both forms timed: refined (FP64 operators) and mixed (FP32 operators)
    timed = {}
    for fname, form in (("refined", bem.FORM_REFINED), ("mixed", bem.FORM_MIXED)):
        launches0 = ctx.kernel_launches
        fms, fclk = _timed_region(args, local, lambda: step(form), stream)
        timed[fname] = {"ms": fms, "clocks": fclk,
                        "gpu_launches": (ctx.kernel_launches - launches0) * args.steps //
                                        (args.steps + max(args.warmup, 3)),
                        "iterations": [reps2[i].iterations for i in range(R * nf)],
                        "fields": [o.copy() for o in outs]}
    refined_fields = timed["refined"]["fields"]
    mixed_fields = timed["mixed"]["fields"]

    # reference: the FP64 operators solved to backward error 1e-12, each wave
    # as its own input
    ref_fields = []
    for d in (with_tol(pw, 1e-12), with_tol(ps, 1e-12)):
        p1 = bem.PreData.from_dict(d, ctx=ctx)
        o = np.zeros((nf, nfp), dtype=np.complex128)
        ctx.check(ctx.lib.bem_run(ctx.h, p1.h, bem.FORM_REFINED, 3, bem._ptr(o), bem._ptr(inc[:nf]),
                                  (bem.SolveReport * nf)(), 0))
        ref_fields.append(o)
        del p1

    def rel(a, b):
        return [float(np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i])) for i in range(nf)]

    err_refined = rel(refined_fields[0], ref_fields[0]) + rel(refined_fields[1], ref_fields[1])
    err_mixed = rel(mixed_fields[0], ref_fields[0]) + rel(mixed_fields[1], ref_fields[1])
    # the headline: the faster form whose every solve is within 1e-6
    best = "mixed" if (max(err_mixed) <= 1e-6 and timed["mixed"]["ms"] < timed["refined"]["ms"]) else "refined"
    ms, clk = timed[best]["ms"], timed[best]["clocks"]
    gpu_launches = timed[best]["gpu_launches"]
    iters = timed[best]["iterations"]
    value = world * nsolve * 1000.0 / ms
    errs_best = err_mixed if best == "mixed" else err_refined

    # end to end through the public API (JSON text + mesh file on the host)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in texts:
        a = bem.Analysis(ctx)
        a.input_from_string(t)
        a.run(form=best, precond="lu")
    e2e_ms = (time.perf_counter() - t0) * 1000.0

    # plain FP64 drop-in form (the reference's H-matrix solver), plane wave only
    plain = None
    if not args.no_plain:
        r = (bem.SolveReport * nf)()
        o = np.zeros((nf, nfp), dtype=np.complex128)
        p1 = bem.PreData.from_dict(pw, ctx=ctx)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.check(ctx.lib.bem_run(ctx.h, p1.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(o), bem._ptr(inc), r, 0))
        torch.cuda.synchronize()
        pms = (time.perf_counter() - t0) * 1000.0
        plain = {"value": nf * 1000.0 / pms, "unit": UNIT, "ms_per_step": pms,
                 "iterations": [r[i].iterations for i in range(nf)],
                 "converged": [r[i].flag == 1 for i in range(nf)],
                 "rel_err": rel(o, ref_fields[0]), "note": "plane-wave input, H-matrix leaf 64, eta 1, ACA 1e-5, "
                                                           "GMRES tol 1e-6 as the input asks"}
        del p1

    ctx.set_profiling(True)
    ctx.check(ctx.lib.bem_run(ctx.h, pds[0].h, bem.FORM_REFINED if best == "refined" else bem.FORM_MIXED, 3,
                              bem._ptr(out2), bem._ptr(inc), (bem.SolveReport * (R * nf))(), 0))
    prof = ctx.profile()
    ctx.set_profiling(False)
    roofline = lu_roofline(prof, [pds[0].n], "8 frequencies of the 40960-unknown ellipsoid")
    threads = max((os.cpu_count() or 2) // 2, 2)
    coarse = workloads.ellipsoid_bm(workdir, n_lon=64, n_bands=21)[0]
    cv, cdt, sample = cpu_reference(coarse, 1, threads)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("fp64" if best == "refined" else "fp32") + " operator / tf32 LU preconditioner (complex)",
        "data": "synthetic (UV ellipsoid mesh, seeded wave direction, no dataset)",
        "config": {"workload": "ellipsoid_bm", "n_unknowns": pds[0].n, "frequencies": nf, "rhs": 2,
                   "ka_a2": [2.5, 20.0],
                   "form": ("refined (FP64 operators)" if best == "refined" else "mixed (FP32 operators)") +
                           " + LU preconditioner, both waves per operator (additional_incident_waves); the faster "
                           "of mixed and refined whose every solve is within 1e-6",
                   "solver": "GMRES tol 1e-8 (input: Hierarchical tol 1e-6)", "parallelism": "replicas only"},
        "e2e": {"value": world * nsolve * 1000.0 / e2e_ms, "unit": UNIT,
                "h2d_bytes_per_step": sum(8 * 3 * pd.info["mesh_nodes"] + 8 * 5 * pd.n + 8 * 3 * pd.nfp for pd in pds),
                "d2h_bytes_per_step": 16 * 2 * nsolve * nfp, "note": "JSON text + VTK file on host -> results on host"},
        "gpu_launches": gpu_launches, "roofline": roofline,
        "cpu_baseline": {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample + "; a 2560-triangle ellipsoid of the same shape (the oracle's H-matrix "
                                            "solve of 40960 unknowns does not fit a bounded sample)"},
        "clocks": clk,
        "by_form": {f: {"value": nsolve * 1000.0 / timed[f]["ms"], "unit": UNIT, "ms_per_step": timed[f]["ms"],
                        "max_rel_err": max(err_mixed if f == "mixed" else err_refined),
                        "iterations": timed[f]["iterations"]} for f in timed},
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
        "rel_err_vs_fp64_reference": errs_best, "max_rel_err_vs_fp64_reference": max(errs_best),
        "error_reference": "field values of the FP64 operators solved to backward error 1e-12",
        "gmres_iterations": iters,
        "stages_ms": {k: v["ms"] for k, v in prof.items()},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def _reference_arm_generic(args, inp, workload, cfg):
    rank, world, local = dist_env()
    if rank != 0:
        return
    threads = max((os.cpu_count() or 2) // 2, 2)
    vals, t_total, sample = [], 0.0, ""
    for _ in range(max(args.steps, 1)):
        v, dt, sample = cpu_reference(inp, 1, threads)
        vals.append(v)
        t_total += dt
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 complex",
            "data": "synthetic", "config": dict(cfg, workload=workload, parallelism="replicas only"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample + " per step; oracle/ C restatement of the reference"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

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
    ap.add_argument("--form", default="mixed", choices=["mixed", "refined", "mixed_rounded"],
                    help="--profile-only: the batched form to run")
    ap.add_argument("--hierarchical", action="store_true",
                    help="with --profile-only: the H-matrix operators (leaf 64, eta 1, ACA 1e-5) instead of dense")
    ap.add_argument("--workload", default=WORKLOAD,
                    choices=[WORKLOAD, "perturbed_spheres", "held_out_learned", "ellipsoid_bm"],
                    help="rigid_sphere_bm (the metric's configuration, default); perturbed_spheres (bodies of "
                         "500-5000 triangles x 8 frequencies in one batch); held_out_learned (learned vs "
                         "block-Jacobi on a held-out 20000-triangle body); ellipsoid_bm (40960 triangles, "
                         "two right-hand sides, 8 frequencies up to ka 20)")
    ap.add_argument("--bodies", type=int, default=256, help="perturbed_spheres: number of bodies")
    ap.add_argument("--train-bodies", type=int, default=16, help="held_out_learned: training bodies")
    ap.add_argument("--train-steps", type=int, default=1000, help="learned preconditioner: training steps")
    ap.add_argument("--held-out-tri", type=int, default=20000, help="held_out_learned: triangles")
    ap.add_argument("--targets", default="all",
                    help="target workloads added to the default line at N = 1 under 'targets': all, none, or a "
                         "comma list of perturbed_spheres, held_out_learned, ellipsoid_bm")
    ap.add_argument("--target-steps", type=int, default=3, help="timed steps per form of each target")
    ap.add_argument("--target-warmup", type=int, default=3, help="warm-up steps per form of each target")
    ap.add_argument("--no-hmatrix", action="store_true", help="ellipsoid target: skip the H-matrix form")
    return ap.parse_args()


def relaunch_as_replicas(nproc, script, argv):
    """`bench.py --gpus N` started without torchrun: run `script` as N ranks
    (one per GPU) under torch.distributed.run on this node, rendezvous on
    127.0.0.1, and return the launcher's exit status."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(nproc),
           "--master-addr", "127.0.0.1", "--master-port", str(port), script] + list(argv)
    return subprocess.call(cmd)


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


def tensor_peak():
    """Dense 16-bit tensor throughput for the FP16 trailing update: the
    sustained cuBLAS BF16 figure of MEASURED_PEAKS.json (FP16 and BF16 run at
    one rate; the trailing updates run for seconds inside the factorization),
    else the fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if d.get("bf16_tflops_sustained"):
            return float(d["bf16_tflops_sustained"]), "measured (cuBLAS BF16 8192^3, sustained)"
    return 1700.0, "fallback (sustained BF16)"


def lu_traffic_ratio(group=4):
    """DRAM traffic / algorithmic A22 bytes of one trailing update over a group
    of four (K = 1024) or eight (K = 2048) block steps, from the committed ncu
    summary (profiles/)."""
    p = os.path.join(ROOT, "profiles", "lu_gemm_trail_group_rigid_sphere.md")
    if not os.path.exists(p):
        return None
    key = "traffic_over_algorithmic:" if group == 4 else "traffic_over_algorithmic_k2048:"
    for line in open(p):
        if line.startswith(key):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def lu_roofline(prof, sizes, what):
    """Roofline entry of the LU preconditioner's trailing update (the dominant
    kernel of the LU forms): flop rate of the trailing-update launches
    (event-timed by the library's profiling pass; 8 n^3 / 3 complex flop per
    factored operator; FP16 operands, FP32 accumulation) against the measured
    dense 16-bit tensor peak.  Block steps run in groups of four (eight from
    12000 unknowns): one K = 1024 (2048) launch per group reads and writes the
    rest of the trailing block once, so its algorithmic bytes are 16 B (FP32
    complex, read + write) per entry of that block (reported per operator: a
    launch covers every operator of a frequency chunk)."""
    lu = prof.get("lu_gemm_trail", {})
    achieved = lu["bytes"] / (lu["ms"] * 1e-3) / 1e12 if lu.get("ms") else None
    peak, peak_kind = tensor_peak()
    # the library's step-group rule: eight steps per pass when every factored
    # system has at least 12000 unknowns
    lb, group = 128, (8 if min(sizes) >= 12000 else 4)
    tot, cnt = 0.0, 0
    for n in sizes:
        nblk = (n + lb - 1) // lb
        for k in range(0, nblk, group):
            m1 = n - (k + group) * lb
            if m1 > 0:
                tot += 16.0 * m1 * m1
                cnt += 1
    alg = tot / cnt if cnt else None
    ratio = lu_traffic_ratio(group)
    return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if achieved else None,
            "traffic": ratio * alg if (ratio and alg) else None,
            "kernel": "lu_gemm_kernel<TRAIL> (FP16 tcgen05 trailing update of the LU preconditioner, " + what + ")",
            "algorithmic_bytes_per_operator_launch": alg,
            "peak_kind": peak_kind,
            "traffic_note": ("ncu dram read+write / algorithmic A22 bytes of one K = %d launch "
                             "(profiles/lu_gemm_trail_group_rigid_sphere.md), times the mean algorithmic bytes "
                             "of this workload's K = %d launches, per operator" % (256 * group, 256 * group))}


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
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_as_replicas(args.gpus, os.path.abspath(__file__), sys.argv[1:]))
    if args.workload in TARGETS:
        if args.impl == "reference":
            return reference_arm_target(args, args.workload)
        return bench_target(args, args.workload)
    rank, world, local = dist_env()
    from cc_abstemious_gb300 import workloads
    workdir = tempfile.mkdtemp(prefix="bem_bench_")
    inp = workloads.rigid_sphere_bm(workdir, m=args.mesh_m, nfreq=args.nfreq)
    if args.profile_only and args.hierarchical:
        # the mixed form over ACA-compressed operators (leaf 64, eta 1, ACA 1e-5)
        inp["solver"] = {"Hierarchical": {"tolerance": 1e-8, "max_iterations": 2500, "leaf_size": 64, "eta": 1.0,
                                          "aca_tolerance": 1e-5}}
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

    form = {"mixed": bem.FORM_MIXED, "refined": bem.FORM_REFINED, "mixed_rounded": bem.FORM_MIXED_ROUNDED}[
        args.form if args.profile_only else "mixed"]

    def run_mixed(check=0):
        ctx.check(ctx.lib.bem_run(ctx.h, pd.h, form, precond, bem._ptr(sc), bem._ptr(inc), reps, check))

    if args.profile_only:
        # the library's per-stage timing runs GMRES iteration by iteration:
        # every kernel is its own launch (a profiler sees them, as it does not
        # inside the solve graph's device-side loop)
        ctx.set_profiling(True)
        run_mixed()
        torch.cuda.synchronize()
        print(json.dumps({k: v["ms"] for k, v in ctx.profile().items()}))
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
    # ---- the target workloads (one GPU): every form, its plain FP64
    # denominator and its error against FP64 LU, one record each
    if world == 1 and args.targets != "none":
        names = list(TARGETS) if args.targets == "all" else [t.strip() for t in args.targets.split(",") if t.strip()]
        del pd
        line["targets"] = run_targets(args, local, names)
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# Target workloads: the configurations the throughput target is stated on
# (perturbed-sphere batch, held-out learned body, ellipsoid).  At N = 1 the
# default line carries one record per target under "targets"; --workload
# prints one target as its own line.  Each record times every form on the
# same resident problem (W warm-up + K timed steps, CUDA events on the library
# stream, clocks sampled meanwhile), measures the plain FP64 denominator with
# the reference's dense solver (FP64 partial-pivot LU, which converges by
# construction), and takes every form's error against an FP64 LU of the same
# operator (the denominator's own solutions where it covers the frequency).

def _timed_region(args, device, fn, stream, steps=None, warmup=None):
    """W warm-up calls, then K calls between CUDA events on the library
    stream, clocks sampled meanwhile; returns (ms per call, clocks)."""
    import torch
    steps = args.steps if steps is None else steps
    warmup = max(args.warmup, 3) if warmup is None else warmup
    for _ in range(warmup):
        fn()
    clocks = Clocks(device)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    return e0.elapsed_time(e1) / steps, clk


def _event_ms(stream, fn):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def _surface(ctx, pd, nrhs, nf):
    """Surface unknowns phi of the last bem_run: (waves, frequencies, n)."""
    import numpy as np
    import cc_abstemious_gb300 as bem
    phi = np.zeros(nrhs * nf * pd.n, dtype=np.complex128)
    ctx.check(ctx.lib.bem_last_surface(ctx.h, pd.h, bem._ptr(phi), None))
    return phi.reshape(nrhs, nf, pd.n)


def _rel(a, b):
    import numpy as np
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _hbm_roofline(prof, what):
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


def _pick_best(forms, tol=1e-6):
    """The fastest form whose every system converged and whose error against
    FP64 LU is within tol."""
    ok = [k for k, v in forms.items() if v.get("converged") and v.get("max_rel_err_vs_fp64_lu") is not None
          and v["max_rel_err_vs_fp64_lu"] <= tol]
    return max(ok, key=lambda k: forms[k]["value"]) if ok else None


class _Shared:
    """What the targets share in one run: the context, its stream, a work
    directory, and the trained network."""

    def __init__(self, args, local):
        import torch
        import cc_abstemious_gb300 as bem
        self.args = args
        self.local = local
        self.ctx = bem.Context(local)
        self.stream = torch.cuda.ExternalStream(self.ctx.stream)
        self.wd = tempfile.mkdtemp(prefix="bem_targets_")
        self.training = None

    def train(self):
        """The learned preconditioner's network, trained on the GPU on
        operators of 16 perturbed spheres drawn like the batch (500-3000
        triangles, ka 0.5..8), once per run."""
        if self.training is not None:
            return self.training
        import numpy as np
        import cc_abstemious_gb300 as bem
        from cc_abstemious_gb300 import workloads
        a = self.args
        train = workloads.perturbed_spheres(self.wd, count=a.train_bodies, seed=1, nfreq=8, tri_lo=500, tri_hi=3000)
        tpds = [bem.PreData.from_dict(d, ctx=self.ctx) for d in train]
        t0 = time.perf_counter()
        losses = bem.learned_train(tpds, steps=a.train_steps, nprobe=8, lr=3e-3, seed=5, ctx=self.ctx)
        self.training = {"bodies": len(train), "steps": a.train_steps, "seconds": time.perf_counter() - t0,
                         "loss_first": float(np.mean(losses[:10])), "loss_last": float(np.mean(losses[-10:]))}
        del tpds
        return self.training

    def lu_roofline(self, prof, sizes, what):
        return lu_roofline(prof, sizes, what)


def target_held_out(sh):
    """Config 5: a held-out perturbed sphere (20000 triangles, ka 4..16 at 12
    frequencies, impedance rho c (1 + 0.2 i), Burton-Miller), the network
    trained on other bodies of the distribution.  Forms: mixed + LU, mixed +
    learned, mixed + block-Jacobi (the method without the network).  GMRES
    stops at backward error 1e-8 (the forward error against FP64 LU stays
    below 1e-6; at 1e-6 it reached 1.3e-6), restart 142 (max_iterations
    20000: at the default 32 the near-field preconditioners stall at ka >= 10)."""
    import numpy as np
    import cc_abstemious_gb300 as bem
    from cc_abstemious_gb300 import workloads
    a, ctx = sh.args, sh.ctx
    training = sh.train()
    kas = np.linspace(4.0, 16.0, 12)
    held = workloads.perturbed_sphere_input(sh.wd, 777777, a.held_out_tri, kas, tol=1e-8)
    held["solver"]["Iterative"]["max_iterations"] = 20000
    pd = bem.PreData.from_dict(held, ctx=ctx)
    # the near-field preconditioners stop at backward error 1e-10: at 1e-8
    # their forward error reached 2e-5 at ka 16 (the LU form overshoots 1e-8
    # by orders in its last iteration and stays near 1e-7)
    tight = json.loads(json.dumps(held))
    tight["solver"]["Iterative"]["tolerance"] = 1e-10
    pd_t = bem.PreData.from_dict(tight, ctx=ctx)
    nf, n = len(pd.frequencies), pd.n
    sc = np.zeros((nf, pd.nfp), dtype=np.complex128)
    inc = np.zeros_like(sc)
    forms = {}
    phis = {}
    for name, form, code, p in (("mixed+lu", bem.FORM_MIXED, 3, pd), ("mixed+learned", bem.FORM_MIXED, 2, pd_t),
                                ("mixed+block_jacobi", bem.FORM_MIXED, 1, pd_t)):
        reps = (bem.SolveReport * nf)()

        def step():
            ctx.check(ctx.lib.bem_run(ctx.h, p.h, form, code, bem._ptr(sc), bem._ptr(inc), reps, 0))

        l0 = ctx.kernel_launches
        ms, clk = _timed_region(a, sh.local, step, sh.stream, a.target_steps, a.target_warmup)
        launches = (ctx.kernel_launches - l0) // (a.target_steps + a.target_warmup)
        phis[name] = _surface(ctx, p, 1, nf)
        forms[name] = {"value": nf * 1000.0 / ms, "unit": UNIT, "ms_per_step": ms, "clocks": clk,
                       "gmres_tol": 1e-8 if p is pd else 1e-10,
                       "gpu_launches": launches, "iterations": [reps[i].iterations for i in range(nf)],
                       "converged": all(reps[i].flag == 1 for i in range(nf)),
                       "precond_used": [reps[i].precond for i in range(nf)]}
    # plain FP64 (the reference's dense solver, partial-pivot LU) at the lowest
    # and highest ka: the denominator and the FP64 LU reference
    idx = [0, nf - 1]
    samp = dict(held, frequency={"List": {"values": [held["frequency"]["List"]["values"][i] for i in idx]}},
                solver={"Direct": {}})
    p2 = bem.PreData.from_dict(samp, ctx=ctx)
    s2 = np.zeros((2, pd.nfp), dtype=np.complex128)
    pms = _event_ms(sh.stream, lambda: ctx.check(ctx.lib.bem_run(ctx.h, p2.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(s2),
                                                                 bem._ptr(s2), None, 0)))
    ref = _surface(ctx, p2, 1, 2)
    plain = {"value": 2 * 1000.0 / pms, "unit": UNIT, "ms": pms,
             "form": "plain FP64, Direct solver (FP64 partial-pivot LU): FP64 assembly + LU + solve + field",
             "sample": "ka %.1f and %.1f (2 of the 12 frequencies)" % (kas[0], kas[-1]), "converged": True}
    for name in forms:
        errs = {"ka%.2f" % kas[i]: _rel(phis[name][0, i], ref[0, j]) for j, i in enumerate(idx)}
        forms[name]["rel_err_vs_fp64_lu"] = errs
        forms[name]["max_rel_err_vs_fp64_lu"] = max(errs.values())
    best = _pick_best(forms)
    code = {"mixed+lu": 3, "mixed+learned": 2, "mixed+block_jacobi": 1}[best or "mixed+lu"]
    ctx.set_profiling(True)
    ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_MIXED, code, bem._ptr(sc), bem._ptr(inc),
                              (bem.SolveReport * nf)(), 0))
    prof = ctx.profile()
    ctx.set_profiling(False)
    roofline = (sh.lu_roofline(prof, [n], "12 frequencies of the held-out body") if code == 3 else
                _hbm_roofline(prof, "12 frequencies of the held-out body"))
    learned, bj = forms["mixed+learned"], forms["mixed+block_jacobi"]
    return {
        "workload": "held_out_learned", "value": forms[best]["value"] if best else None, "unit": UNIT,
        "best_form": best, "steps": a.target_steps, "warmup": a.target_warmup,
        "config": {"n_unknowns": n, "frequencies": nf, "ka": [4.0, 16.0], "bc": "impedance rho c (1 + 0.2i)",
                   "solver": "GMRES backward error 1e-8 (LU form) or 1e-10 (near-field preconditioners), "
                             "restart 142", "training": training},
        "forms": forms, "plain_fp64": plain,
        "speedup_vs_plain_fp64": forms[best]["value"] / plain["value"] if best else None,
        "learned_vs_plain_fp64": learned["value"] / plain["value"],
        "learned_vs_block_jacobi": {"solves_per_s": learned["value"] / bj["value"],
                                    "iterations": [sum(learned["iterations"]), sum(bj["iterations"])]},
        "max_rel_err_vs_fp64_lu": forms[best]["max_rel_err_vs_fp64_lu"] if best else None,
        "roofline": roofline, "stages_ms": {k: v["ms"] for k, v in prof.items()},
    }


def target_perturbed_spheres(sh):
    """Config 4: 256 harmonic-perturbed spheres (500-5000 triangles each,
    impedance rho c (1 + 0.2 i), Burton-Miller, ka 0.5..8 at 8 frequencies),
    every body and frequency in one batch (bem_run_batch).  Forms: mixed +
    LU, mixed + learned, mixed + block-Jacobi; GMRES tol 1e-8 (backward
    error), restart 71.  The plain FP64 denominator is the reference's dense
    solver on a stated sample of the bodies (every 16th)."""
    import numpy as np
    import cc_abstemious_gb300 as bem
    from cc_abstemious_gb300 import workloads
    a, ctx = sh.args, sh.ctx
    training = sh.train()
    inps = workloads.perturbed_spheres(sh.wd, count=a.bodies, seed=0, nfreq=8, tol=1e-8)
    for d in inps:
        d["solver"]["Iterative"]["max_iterations"] = 5000
    pds = [bem.PreData.from_dict(d, ctx=ctx) for d in inps]
    ns = [pd.n for pd in pds]
    nsys = sum(len(pd.frequencies) for pd in pds)
    order = np.argsort(ns)
    pick = sorted({int(order[0]), int(order[len(order) // 2]), int(order[-1])})
    forms = {}
    last = {}
    for name, pc in (("mixed+lu", "lu"), ("mixed+learned", "learned"), ("mixed+block_jacobi", "block_jacobi")):
        def step():
            last["out"] = bem.run_batch(pds, precond=pc, ctx=ctx)

        l0 = ctx.kernel_launches
        ms, clk = _timed_region(a, sh.local, step, sh.stream, a.target_steps, a.target_warmup)
        launches = (ctx.kernel_launches - l0) // (a.target_steps + a.target_warmup)
        its = [r["iterations"] for _, reps in last["out"] for r in reps]
        conv = all(r["flag"] == 1 for _, reps in last["out"] for r in reps)
        chk = bem.run_batch([pds[i] for i in pick], precond=pc, check_vs_lu=True, ctx=ctx)
        errs = {"body%d_N%d" % (i, ns[i]): max(r["rel_err_vs_lu"] for r in reps) for i, (_, reps) in zip(pick, chk)}
        forms[name] = {"value": nsys * 1000.0 / ms, "unit": UNIT, "ms_per_step": ms, "clocks": clk,
                       "gpu_launches": launches, "iterations_mean": float(np.mean(its)),
                       "iterations_max": int(max(its)), "converged": conv, "rel_err_vs_fp64_lu": errs,
                       "max_rel_err_vs_fp64_lu": max(errs.values())}
    # plain FP64: the reference's dense solver (partial-pivot LU), body by body
    sample = list(range(0, len(inps), 16))
    p2 = [bem.PreData.from_dict(dict(inps[i], solver={"Direct": {}}), ctx=ctx) for i in sample]
    s2 = np.zeros((8, pds[0].nfp), dtype=np.complex128)

    def plain_all():
        for p in p2:
            ctx.check(ctx.lib.bem_run(ctx.h, p.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(s2), bem._ptr(s2), None, 0))

    pms = _event_ms(sh.stream, plain_all)
    nplain = sum(len(p.frequencies) for p in p2)
    plain = {"value": nplain * 1000.0 / pms, "unit": UNIT, "ms": pms,
             "form": "plain FP64, Direct solver (FP64 partial-pivot LU), body by body",
             "sample": "%d of the %d bodies (every 16th in generation order, sizes %d-%d), all 8 frequencies" % (
                 len(sample), len(inps), min(ns[i] for i in sample), max(ns[i] for i in sample)),
             "converged": True}
    del p2
    best = _pick_best(forms)
    ctx.set_profiling(True)
    bem.run_batch(pds, precond={"mixed+lu": "lu", "mixed+learned": "learned",
                                "mixed+block_jacobi": "block_jacobi"}[best or "mixed+lu"], ctx=ctx)
    prof = ctx.profile()
    ctx.set_profiling(False)
    roofline = (sh.lu_roofline(prof, list(ns), "ragged batch over all bodies and frequencies")
                if best in (None, "mixed+lu") else _hbm_roofline(prof, "ragged batch over all bodies"))
    learned, bj = forms["mixed+learned"], forms["mixed+block_jacobi"]
    return {
        "workload": "perturbed_spheres", "value": forms[best]["value"] if best else None, "unit": UNIT,
        "best_form": best, "steps": a.target_steps, "warmup": a.target_warmup,
        "config": {"bodies": len(pds), "frequencies_per_body": 8, "systems": nsys, "n_min": int(min(ns)),
                   "n_max": int(max(ns)), "n_mean": float(np.mean(ns)), "ka": [0.5, 8.0],
                   "bc": "impedance rho c (1 + 0.2i)", "solver": "GMRES tol 1e-8 (backward error), restart 71",
                   "training": training,
                   "l2": "operators %.1f GB > L2 (no flush needed)" % (8e-9 * sum(
                       (-(-pd.n // 64) * 64) * pd.n * len(pd.frequencies) for pd in pds))},
        "forms": forms, "plain_fp64": plain,
        "speedup_vs_plain_fp64": forms[best]["value"] / plain["value"] if best else None,
        "learned_vs_plain_fp64": learned["value"] / plain["value"],
        "learned_vs_block_jacobi": {"solves_per_s": learned["value"] / bj["value"],
                                    "iterations_mean": [learned["iterations_mean"], bj["iterations_mean"]]},
        "max_rel_err_vs_fp64_lu": forms[best]["max_rel_err_vs_fp64_lu"] if best else None,
        "roofline": roofline, "stages_ms": {k: v["ms"] for k, v in prof.items()},
    }


def target_ellipsoid(sh):
    """Config 3: ellipsoid (2, 1, 0.5) m with 40960 triangles, Burton-Miller,
    a plane wave along a seeded direction and a point source at (0, 0, 3),
    ka (a = 2) 2.5..20 at 8 frequencies: 16 solves per step.  The forms solve
    the dense operators with the tensor-core LU preconditioner, both waves per
    operator (extension key additional_incident_waves), GMRES at backward
    error 1e-8, in order of cost until one meets 1e-6: mixed (FP32 operators
    of the single-precision assembly), mixed_rounded (FP32 operators rounded
    once from float-float values) and refined (operators at FP64 accuracy).  The plain FP64 denominator and the error
    reference are the reference's dense solver (FP64 partial-pivot LU, both
    waves from one factorization) at the lowest and highest ka."""
    import numpy as np
    import cc_abstemious_gb300 as bem
    from cc_abstemious_gb300 import workloads
    a, ctx = sh.args, sh.ctx
    pw, ps = workloads.ellipsoid_bm(sh.wd)
    both = json.loads(json.dumps(pw))
    both["solver"] = {"Iterative": {"tolerance": 1e-8, "max_iterations": 1000}}
    both["additional_incident_waves"] = [ps["incident_wave"]]
    pd = bem.PreData.from_dict(both, ctx=ctx)
    nf, n, R = len(pd.frequencies), pd.n, 2
    out = np.zeros((R * nf, pd.nfp), dtype=np.complex128)
    inc = np.zeros_like(out)
    # FP64 LU reference and plain denominator first (the forms' operators
    # then reuse the same device memory)
    idx = [0, nf - 1]
    freqs = both["frequency"]["List"]["values"]
    samp = dict(both, frequency={"List": {"values": [freqs[i] for i in idx]}}, solver={"Direct": {}})
    p2 = bem.PreData.from_dict(samp, ctx=ctx)
    s2 = np.zeros((R * 2, pd.nfp), dtype=np.complex128)
    pms = _event_ms(sh.stream, lambda: ctx.check(ctx.lib.bem_run(ctx.h, p2.h, bem.FORM_PLAIN_FP64, 0, bem._ptr(s2),
                                                                 bem._ptr(s2), None, 0)))
    ref = _surface(ctx, p2, R, 2)
    del p2
    kas = np.linspace(2.5, 20.0, nf)
    plain = {"value": R * 2 * 1000.0 / pms, "unit": UNIT, "ms": pms,
             "form": "plain FP64, Direct solver (FP64 partial-pivot LU, both waves from one factorization): "
                     "FP64 assembly + LU + solves + field",
             "sample": "ka %.1f and %.1f (2 of the 8 frequencies), both waves" % (kas[0], kas[-1]),
             "converged": True,
             "note": "the input's own solver (H-matrix, leaf 64, eta 1, ACA 1e-5, GMRES(32) tol 1e-6) does not "
                     "converge on this body (992 iterations at every frequency)"}
    forms = {}
    codes = {"mixed+lu": bem.FORM_MIXED, "mixed_rounded+lu": bem.FORM_MIXED_ROUNDED, "refined+lu": bem.FORM_REFINED}
    for name, form in codes.items():
        reps = (bem.SolveReport * (R * nf))()

        def step():
            ctx.check(ctx.lib.bem_run(ctx.h, pd.h, form, 3, bem._ptr(out), bem._ptr(inc), reps, 0))

        l0 = ctx.kernel_launches
        ms, clk = _timed_region(a, sh.local, step, sh.stream, a.target_steps, a.target_warmup)
        launches = (ctx.kernel_launches - l0) // (a.target_steps + a.target_warmup)
        phi = _surface(ctx, pd, R, nf)
        errs = {"wave%d_ka%.1f" % (r, kas[i]): _rel(phi[r, i], ref[r, j]) for r in range(R)
                for j, i in enumerate(idx)}
        forms[name] = {"value": R * nf * 1000.0 / ms, "unit": UNIT, "ms_per_step": ms, "clocks": clk,
                       "gpu_launches": launches, "iterations": [reps[i].iterations for i in range(R * nf)],
                       "converged": all(reps[i].flag == 1 for i in range(R * nf)), "rel_err_vs_fp64_lu": errs,
                       "max_rel_err_vs_fp64_lu": max(errs.values())}
        if forms[name]["converged"] and forms[name]["max_rel_err_vs_fp64_lu"] <= 1e-6:
            break  # the costlier forms are only needed when this one misses 1e-6
    best = _pick_best(forms)
    ctx.set_profiling(True)
    ctx.check(ctx.lib.bem_run(ctx.h, pd.h, codes[best or "refined+lu"], 3,
                              bem._ptr(out), bem._ptr(inc), (bem.SolveReport * (R * nf))(), 0))
    prof = ctx.profile()
    ctx.set_profiling(False)
    hmat = None if a.no_hmatrix else _ellipsoid_hmatrix(sh, samp, R, idx, kas, ref)
    return {
        "workload": "ellipsoid_bm", "value": forms[best]["value"] if best else None, "unit": UNIT,
        "best_form": best, "steps": a.target_steps, "warmup": a.target_warmup,
        "config": {"n_unknowns": n, "frequencies": nf, "rhs": R, "ka_a2": [2.5, 20.0],
                   "solver": "GMRES tol 1e-8 (backward error) with the LU preconditioner, dense operators "
                             "(input: Hierarchical tol 1e-6)",
                   "learned": "not in the timed forms: measured separately (bench's network, mixed form, both "
                              "waves, GMRES tol 1e-8 up to 20000 iterations), the near-field learned and "
                              "block-Jacobi preconditioners do not converge at ka 2.5 (20000 iterations, 91 s "
                              "per frequency) and take 424-620 iterations at ka 20, the learned one the same "
                              "count as block-Jacobi; the LU preconditioner takes 4-6"},
        "forms": forms, "plain_fp64": plain,
        "speedup_vs_plain_fp64": forms[best]["value"] / plain["value"] if best else None,
        "max_rel_err_vs_fp64_lu": forms[best]["max_rel_err_vs_fp64_lu"] if best else None,
        "roofline": sh.lu_roofline(prof, [n], "8 frequencies of the 40960-unknown ellipsoid"),
        "stages_ms": {k: v["ms"] for k, v in prof.items()},
        "hmatrix_form": hmat,
    }


def _ellipsoid_hmatrix(sh, samp, R, idx, kas, ref):
    """The input's own solver in the mixed form: ACA-compressed operators (leaf
    64, eta 1, ACA 1e-5) with FP32 factors, block-Jacobi on the diagonal
    leaves, GMRES backward error 1e-8 within 4000 iterations, at the sampled
    frequencies (both waves).  One warm-up and one timed step (a step builds
    every operator by ACA in FP64, which dominates); the roofline is its
    mat-vec's stored bytes over the event-timed launches against the copy
    bandwidth."""
    import numpy as np
    import cc_abstemious_gb300 as bem
    ctx = sh.ctx
    hm = json.loads(json.dumps(samp))
    hm["solver"] = {"Hierarchical": {"tolerance": 1e-8, "max_iterations": 4000, "leaf_size": 64, "eta": 1.0,
                                     "aca_tolerance": 1e-5}}
    pd = bem.PreData.from_dict(hm, ctx=ctx)
    nf = len(pd.frequencies)
    out = np.zeros((R * nf, pd.nfp), dtype=np.complex128)
    reps = (bem.SolveReport * (R * nf))()

    def step():
        ctx.check(ctx.lib.bem_run(ctx.h, pd.h, bem.FORM_MIXED, 1, bem._ptr(out), bem._ptr(out), reps, 0))

    ms, clk = _timed_region(sh.args, sh.local, step, sh.stream, 1, 1)
    phi = _surface(ctx, pd, R, nf)
    conv = [reps[i].flag == 1 for i in range(R * nf)]
    errs = {"wave%d_ka%.1f" % (r, kas[i]): _rel(phi[r, j], ref[r, j]) for r in range(R) for j, i in enumerate(idx)}
    ctx.set_profiling(True)
    step()
    prof = ctx.profile()
    ctx.set_profiling(False)
    hbm_peak, peak_kind = measured_peaks()
    mv = prof.get("gmres_matvec_hmatrix", {})
    build = prof.get("hmatrix_build", {})
    achieved = mv["bytes"] / (mv["ms"] * 1e-3) / 1e9 if mv.get("ms") else None
    stored = build.get("bytes", 0.0) / 8.0
    return {"form": "mixed over H-matrix operators (Hierarchical solver), block-Jacobi", "steps": 1, "warmup": 1,
            "value": R * nf * 1000.0 / ms, "unit": UNIT, "ms_per_step": ms, "clocks": clk,
            "sample": "ka %.1f and %.1f, both waves" % (kas[idx[0]], kas[idx[-1]]),
            "iterations": [reps[i].iterations for i in range(R * nf)], "converged": conv,
            "rel_err_vs_fp64_lu": errs, "max_rel_err_vs_fp64_lu": max(errs.values()),
            "error_note": "against the FP64 LU of the dense operator: includes the ACA error (tolerance 1e-5)",
            "stored_complex_entries_per_operator": stored / nf,
            "dense_entries_per_operator": float(pd.n) * pd.n,
            "stages_ms": {k: v["ms"] for k, v in prof.items()},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak if achieved else None, "traffic": None,
                         "kernel": "hmx_project_kernel + hmx_rows_kernel (H-matrix Krylov mat-vec, FP32 factors)",
                         "algorithmic_bytes_per_launch": mv["bytes"] / max(mv["launches"], 1) if mv else None,
                         "peak_kind": peak_kind + " (burst copy)"}}


def reference_arm_target(args, name):
    """--impl reference --workload <target>: the oracle (C restatement of the
    reference algorithm) on a bounded sample of that workload, host cores."""
    from cc_abstemious_gb300 import workloads
    import numpy as np
    rank, world, local = dist_env()
    if rank != 0:
        return
    wd = tempfile.mkdtemp(prefix="bem_ref_")
    if name == "perturbed_spheres":
        inps = workloads.perturbed_spheres(wd, count=args.bodies, seed=0, nfreq=8, tol=1e-8)
        inp, what = inps[len(inps) // 2], "body %d of the batch" % (len(inps) // 2)
    elif name == "held_out_learned":
        inp = workloads.perturbed_sphere_input(wd, 777777, 2000, np.linspace(4.0, 16.0, 12), tol=1e-8)
        what = "a 2000-triangle body of the held-out distribution (20000 triangles do not fit a bounded sample)"
    else:
        inp = workloads.ellipsoid_bm(wd, n_lon=64, n_bands=21)[0]
        what = "a 2560-triangle ellipsoid of the same shape (40960 triangles do not fit a bounded sample)"
    threads = max((os.cpu_count() or 2) // 2, 2)
    for _ in range(args.warmup):
        cpu_reference(inp, 1, threads)
    vals, t_total, sample = [], 0.0, ""
    for _ in range(max(args.steps, 1)):
        v, dt, sample = cpu_reference(inp, 1, threads)
        vals.append(v)
        t_total += dt
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 complex",
            "data": "synthetic", "config": {"workload": name, "parallelism": "replicas only"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample + "; " + what + "; oracle/ C restatement of the reference"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


TARGETS = {"perturbed_spheres": target_perturbed_spheres, "held_out_learned": target_held_out,
           "ellipsoid_bm": target_ellipsoid}


def run_targets(args, local, names):
    """Every named target on a fresh context; a target that fails is
    reported with its error instead of stopping the run."""
    import torch
    sh = _Shared(args, local)
    out = {}
    for name in names:
        t0 = time.perf_counter()
        try:
            out[name] = TARGETS[name](sh)
        except Exception as e:  # noqa: BLE001 -- reported in the line
            out[name] = {"workload": name, "error": "%s: %s" % (type(e).__name__, e)}
        out[name]["wall_s"] = time.perf_counter() - t0
        torch.cuda.synchronize()
    return out


def bench_target(args, name):
    """--workload <target>: that target's record as its own line, with the
    contract's keys at the top."""
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    rec = run_targets(args, local, [name])[name]
    best = rec.get("forms", {}).get(rec.get("best_form") or "", {})
    line = {"metric": METRIC, "value": rec.get("value"), "unit": UNIT, "n_gpus": 1,
            "steps": rec.get("steps"), "warmup": rec.get("warmup"), "ms_per_step": best.get("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 operator / fp64 vectors (complex)", "data": "synthetic (seeded meshes, no dataset)",
            "config": {"workload": name, "parallelism": "replicas only"}, "gpu_launches": best.get("gpu_launches"),
            "clocks": best.get("clocks"), "target": rec}
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

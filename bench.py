"""Benchmark: load steps/s of the 1M-particle SC elastoplastic cyclic case.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one load step of src/lpmc_project.c:385-471): simple
cubic lattice 100 x 100 x 100 (1e6 particles, 8.9e6 bonds, 3e6 DOF),
spacing 0.2 mm, E = 200 GPa with +-5% uniform noise per particle (seed 1),
nu = 0.3, J2 yield 250 MPa, linear hardening 2 GPa; bottom face fixed in z
(plus a 3-DOF rigid-body pin), top face displaced along the +-0.2% strain
cycle, 20 steps per quarter cycle; Newton tolerance 1e-8 with the
reference's MAXITER of 100, linear solves to relative residual 1e-10.  The W
warm-up steps are the first W steps of the schedule; the K timed steps follow
them (the default 5 + 20 reach through the plastic steps 12-20).

Headline: the mixed-precision path (FP32 stiffness and PCG products in
difference form, FP64 PCG vectors, reliable updates, residuals and return
map) with the multigrid-preconditioned PCG.  The same steps run on the plain
FP64 path for the ratio and the errors between the two.  Inputs are resident
in HBM (value); `e2e` runs the same steps through the reference-named C
drop-in (liblpmhost.so + liblpmgpu_legacy.so) with the include/lpm.h globals
on the host, host<->device copies inside the timed region.  The reference arm
times the oracle's C port of the reference algorithm on the host cores.

Time budget: the arms run in the order mixed, FP64, e2e, CPU baseline; an arm
that would not fit the remaining budget (--budget, from process start) is
skipped and reported as such, and a watchdog prints the line measured so far
at --budget + --grace seconds, so the run always ends with its JSON line.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "lpm-c_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import cases  # noqa: E402

T_START = time.time()

METRIC = "load steps/s, 1M-particle SC lattice: mixed vs FP64 GPU @1e-8 err; SpMV GB/s"
UNIT = "load steps/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, device=None):
    """Max of a per-rank float over the process group (identity on one rank)."""
    try:
        import torch
        import torch.distributed as dist
    except Exception:
        return value
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.tmp.close()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        loaded = sorted(sm)[len(sm) // 2:] if sm else []
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows)}


def build_specimen(G, case, precision, stream=None, precond=0):
    s = G.Specimen(0)
    if stream is not None:
        s.set_stream(stream)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(s.get("xyz"), s.get("nb"), case.radius)
    s.set_types(types)
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    u = cases.splitmix64_uniform(case.seed, n)
    sc = 1.0 + case.e_noise * (2.0 * u - 1.0)
    s.set_material(c11 * sc, c12 * sc, c44 * sc, case.sigmay, case.H, 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(**solver_opts(G, case, precision, precond))
    return s, types


def solver_opts(G, case, precision, precond):
    """Newton tolerance 1e-8 and the reference's MAXITER of 100
    (include/lpm.h:39), linear solves to 1e-10 relative.  The multigrid PCG
    needs about 40 iterations per solve: its cap of 2000 bounds the time a
    misbehaving solve can take.  Each Newton solve of a step starts from the
    Galerkin combination of the step's last 8 solutions (recycle), in both
    precisions."""
    return dict(precision=precision, newton_tol=case.newton_tol, newton_maxiter=100, cg_rtol=CG_RTOL,
                cg_maxiter=2000 if precond else 200000, preconditioner=precond, recycle=RECYCLE)


RECYCLE = 8  # earlier solutions of the load step the Newton solves start from
CG_RTOL = 1e-10  # relative residual of the SC workload's linear solves (--cg-rtol)
DIFF_STREAM = -1  # form of the mixed multigrid product (--diff-stream; -1: the autotuner's choice)
SMOOTH_STREAM = -1  # form of the multigrid level-0 smoother (--smooth-stream; -1: the autotuner's choice)


class Deadline:
    """Wall-clock budget of the whole run, counted from process start."""

    def __init__(self, budget_s):
        self.t_end = T_START + budget_s

    def left(self):
        return self.t_end - time.time()


def run_arm(G, case, prec, precond, W, K, stream, deadline, sync, autotune=True):
    """One precision on the SC workload: setup, W warm-up load steps, then K
    timed load steps bracketed by CUDA events on the launching stream.  Stops
    between steps once the deadline has passed (the arm then reports
    incomplete, never fewer steps)."""
    import torch
    t0 = time.time()
    s, types = build_specimen(G, case, prec, stream.cuda_stream, precond)
    setup_s = time.time() - t0
    sched = case.schedule
    tuning = None
    warm = []
    for k in range(W):
        if deadline.left() < 0:
            s.close()
            return {"incomplete": f"deadline passed in warm-up step {k + 1}"}
        warm.append(s.load_step(cases.sc_bcs(sched[k])))
        if k == 0 and autotune:
            tuning = s.autotune()  # launch shapes from the project's autotuner
        if k == 0 and precond and (DIFF_STREAM >= 0 or SMOOTH_STREAM >= 0):
            t = s.get_tuning()
            ds = DIFF_STREAM if (DIFF_STREAM >= 0 and prec == G.PREC_MIXED) else t["diff_stream"]
            ss = SMOOTH_STREAM if SMOOTH_STREAM >= 0 else t["smooth_stream"]
            s.set_tuning(spmv_variant=t["spmv_variant"], spmv_per_sm=t["spmv_per_sm"], cg_per_sm=t["cg_per_sm"],
                         diff_stream=ds, smooth_stream=ss)
            tuning = dict(tuning or {}, diff_stream=ds, smooth_stream=ss, set_by="--diff-stream/--smooth-stream")
    sync()
    s.spmv_timing(reset=2)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    wall = []
    sync()
    ev0.record(stream)
    for k in range(W, W + K):
        if deadline.left() < 0:
            ev1.record(stream)
            sync()
            clocks.stop()
            s.close()
            return {"incomplete": f"deadline passed before timed step {k + 1} ({k - W} of {K} done)",
                    "stats": stats}
        t1 = time.time()
        stats.append(s.load_step(cases.sc_bcs(sched[k])))
        wall.append(time.time() - t1)
    ev1.record(stream)
    sync()
    ms = ev0.elapsed_time(ev1)
    ck = clocks.stop()
    spmv_ms, spmv_cnt = s.spmv_timing(reset=3)
    out = dict(ms=ms, stats=stats, warm=warm, spmv_ms=spmv_ms, spmv_cnt=spmv_cnt, clocks=ck, tuning=tuning,
               spmv_bytes=spmv_alg_bytes(s, prec, precond), xyz=s.get("xyz"), x0=s.get("xyz_initial"),
               alpha=s.get("J2_alpha"), react=reaction(s, types), n=s.n, nnzb=s.sizes()["nnz_blocks"],
               setup_s=setup_s, step_wall_s=wall)
    s.close()
    return out


def reaction(s, types):
    """Reaction of the top face, writeReaction's sum of -cs_z F over the
    particles of the type (src/data_handler.c:309-335)."""
    top = types == cases.T_TOP
    return float(np.sum(-s.get("csz")[top] * s.get("F")[top]))


def spmv_alg_bytes(s, prec, precond):
    """Algorithmic bytes of one launch of the PCG product the arm runs: the
    stiffness values and column indices of the structural (unpadded) blocks,
    the row offsets, the input vector read once and the output written once.
    FP64: 72 B of values per block, FP64 vectors (24 B per particle each way).
    Mixed with the multigrid: the difference-form FP32 product, 36 B of values
    per block, the input as two FP32 parts (24 B per particle), the FP64 output
    (24 B) and the 3 x 3 block row sums (36 B per particle).  Mixed with
    block-Jacobi: the FP32 SpMV on FP32 vectors (12 B each way)."""
    z = s.sizes()
    nnzb, n = z["nnz_blocks"], s.n
    if prec == 0:
        return nnzb * (9 * 8 + 4) + 4 * (n + 1) + 2 * 3 * n * 8
    if precond:
        return nnzb * (9 * 4 + 4) + 4 * (n + 1) + 3 * n * 8 + 3 * n * 8 + 9 * n * 4
    return s.spmv_bytes(prec)


def run_ours(args):
    import torch
    import lpm_gb300 as G
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    case = cases.SCCase(n=args.size, e_noise=0.05, seed=1)
    W, K = args.warmup, args.steps
    stream = torch.cuda.current_stream()
    precond = G.PRECOND_AMG if args.precond == "amg" else G.PRECOND_BJ
    deadline = Deadline(args.budget)

    def sync():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    state = {"line": None}
    lock = threading.Lock()

    def emit(line):
        with lock:
            if state["line"] is None and rank == 0:
                state["line"] = line
                print(json.dumps(line), flush=True)

    # hard stop: print what has been measured and leave before an outer limit
    # cuts the run off without a line
    partial = {}

    def watchdog():
        emit(assemble_line(args, case, partial, world, note="hard time limit reached; unfinished parts are null"))
        os._exit(0)

    timer = threading.Timer(max(1.0, args.budget + args.grace - (time.time() - T_START)), watchdog)
    timer.daemon = True
    timer.start()

    head_prec = G.PREC_FP64 if args.arm_precision == "fp64" else G.PREC_MIXED
    partial["mixed"] = run_arm(G, case, head_prec, precond, W, K, stream, deadline, sync,
                               autotune=not args.no_autotune)
    mixed = partial["mixed"]
    mixed_s = mixed["ms"] / 1e3 if "ms" in mixed else None
    # the FP64 arm runs the same steps; its FP64 product is about 4x the
    # mixed one's per PCG iteration, so budget it at 3x the mixed arm
    if args.no_fp64:
        partial["fp64"] = {"skipped": "--no-fp64"}
    elif mixed_s is None:
        partial["fp64"] = {"skipped": "the mixed arm did not finish"}
    elif deadline.left() < 3.0 * (mixed_s + mixed["setup_s"]) + 60.0:
        partial["fp64"] = {"skipped": f"budget: {deadline.left():.0f} s left, about {3.0 * mixed_s:.0f} s needed"}
    else:
        partial["fp64"] = run_arm(G, case, G.PREC_FP64, precond, W, K, stream, deadline, sync,
                                  autotune=not args.no_autotune)
    if args.no_e2e or rank != 0:
        partial["e2e"] = None
    elif mixed_s is None:
        partial["e2e"] = {"value": None, "unit": UNIT, "skipped": "the mixed arm did not finish"}
    elif deadline.left() < 2.5 * mixed_s + 60.0:
        partial["e2e"] = {"value": None, "unit": UNIT,
                          "skipped": f"budget: {deadline.left():.0f} s left, about {2.5 * mixed_s:.0f} s needed"}
    else:
        partial["e2e"] = run_e2e(args, case, precond, deadline)
    if args.no_cpu or rank != 0:
        partial["cpu"] = None
    else:
        partial["cpu"] = run_cpu_baseline(case, W, K)
    line = assemble_line(args, case, partial, world)
    timer.cancel()
    emit(line)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def assemble_line(args, case, partial, world, note=None):
    """The JSON line from whatever the arms have measured so far."""
    W, K = args.warmup, args.steps
    mixed = partial.get("mixed") or {}
    f64 = partial.get("fp64") or {}
    done = "ms" in mixed
    value = world * K / (mixed["ms"] / 1e3) if done else None
    hbm, peak_src = peaks()
    achieved = (mixed["spmv_bytes"] / (mixed["spmv_ms"] * 1e-3) / 1e9
                if done and mixed.get("spmv_ms") else None)
    fp64_rate = world * K / (f64["ms"] / 1e3) if "ms" in f64 else None
    errs = {}
    if done and "ms" in f64:
        du_m, du_f = mixed["xyz"] - mixed["x0"], f64["xyz"] - f64["x0"]
        errs["disp_err_mixed_vs_fp64"] = float(np.abs(du_m - du_f).max() / np.abs(du_f).max())
        errs["plastic_strain_err_mixed_vs_fp64"] = float(np.abs(mixed["alpha"] - f64["alpha"]).max() /
                                                         max(np.abs(f64["alpha"]).max(), 1e-300))
        errs["reaction_err_mixed_vs_fp64"] = abs(mixed["react"] - f64["react"]) / abs(f64["react"])
    agg = (lambda arm, key: int(sum(st[key] for st in arm["stats"]))) if True else None  # noqa: E731
    sched_len = len(case.schedule)
    precond_name = ("smoothed-aggregation multigrid V-cycle" if args.precond == "amg" else "block-Jacobi")
    cfg = {"workload": f"SC {args.size}^3 elastoplastic cyclic (E +-5 % per particle), load steps "
                       f"{W + 1}-{W + K} of {sched_len}: first yield at step 12, steps 15-20 stop at the "
                       f"reference's 100 Newton iterations",
           "particles": mixed.get("n"), "nnz_blocks": mixed.get("nnzb"), "precision": "mixed",
           "preconditioner": precond_name,
           "newton": "modified Newton with the elastic tangent of the step (src/lpmc_project.c:382-471), "
                     f"tolerance 1e-8, MAXITER 100; linear solves to {CG_RTOL:g} relative, each started from the "
                     f"Galerkin combination of the step's last {RECYCLE} solutions (both precisions)",
           "fp64_steps_per_s": fp64_rate, "mixed_over_fp64": (value / fp64_rate) if (value and fp64_rate) else None,
           **errs,
           "fp64_arm": {k: v for k, v in f64.items() if k in ("skipped", "incomplete")} or None,
           "newton_iters": agg(mixed, "newton_iters") if done else None,
           "newton_iters_per_step": [st["newton_iters"] for st in mixed["stats"]] if done else None,
           "newton_iters_per_warmup_step": [st["newton_iters"] for st in mixed["warm"]] if done else None,
           "cg_iters_per_step": [st["cg_iters"] for st in mixed["stats"]] if done else None,
           "cg_iters": agg(mixed, "cg_iters") if done else None,
           "reliable_updates": agg(mixed, "refine_iters") if done else None,
           "fp64_newton_iters": agg(f64, "newton_iters") if "ms" in f64 else None,
           "fp64_cg_iters": agg(f64, "cg_iters") if "ms" in f64 else None,
           "step_wall_s": [round(x, 3) for x in mixed["step_wall_s"]] if done else None,
           "l2": "stiffness stream of 2.4 GB (FP32) per product > 129 MB L2 (no flush needed)",
           "tuning": mixed.get("tuning"),
           "amg_build_ms": (sum(st["ms_amg_build"] for st in mixed["warm"] + mixed["stats"]) if done else None),
           "amg_builds": (sum(st["amg_builds"] for st in mixed["warm"] + mixed["stats"]) if done else None),
           "setup_s": mixed.get("setup_s"),
           "parallelism": "replicas" if world > 1 else "single GPU"}
    if not done:
        cfg["mixed_arm"] = {k: v for k, v in mixed.items() if k in ("skipped", "incomplete")}
    if note:
        cfg["note"] = note
    streamed = bool((mixed.get("tuning") or {}).get("diff_stream", 0)) and args.precond == "amg"
    if streamed:
        kernel = ("k_spmv_diff_stream (difference-form FP32 block-CSR product of the mixed multigrid PCG, "
                  "stiffness streamed into shared memory by the bulk-copy engine)")
    elif args.precond == "amg":
        kernel = "k_spmv_diff (difference-form FP32 block-CSR product of the mixed multigrid PCG)"
    else:
        kernel = "k_spmv<float, float4> (FP32 block-CSR SpMV)"
    traffic_ratio = SPMV_STREAM_TRAFFIC_OVER_ALG if streamed else SPMV_TRAFFIC_OVER_ALG
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": (mixed["ms"] / K) if done else None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 stiffness and PCG products + f64 PCG vectors, residuals, reliable updates and return map",
        "data": "synthetic (seeded lattice and per-particle material noise)",
        "config": cfg,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None,
                     "traffic": (mixed["spmv_bytes"] * traffic_ratio) if done else None,
                     "kernel": kernel, "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": mixed.get("spmv_bytes"),
                     "launches_sampled": mixed.get("spmv_cnt")},
        "clocks": mixed.get("clocks"),
        "gpu_launches": gpu_launches(mixed["stats"], amg_levels(mixed["n"]) if args.precond == "amg" else 0)
        if done else None,
        "e2e": partial.get("e2e"),
        "cpu_baseline": partial.get("cpu"),
    }
    return line


# DRAM bytes over algorithmic bytes of the PCG product, from the ncu capture
# of k_spmv_diff at SC 60^3 (dram__bytes_read.sum + dram__bytes_write.sum of
# one launch, 547.11 MB over 519.69 MB; the ncu summary of k_spmv_diff under profiles/),
# applied to the 1M-particle launch
SPMV_TRAFFIC_OVER_ALG = 1.0528
# the same for k_spmv_diff_stream in the autotuner's 8-row shape (549.56 MB over
# 519.69 MB; the ncu summary of k_spmv_diff_stream under profiles/)
SPMV_STREAM_TRAFFIC_OVER_ALG = 1.0575


def amg_levels(n, coarse_blocks=150):
    """Levels above the coarsest of the multigrid hierarchy of a cube of n
    particles (aggregates of 3 x 3 x 3 block rows per level)."""
    m, levels = round(n ** (1.0 / 3.0)), 0
    while m ** 3 > coarse_blocks and levels < 8:
        m, levels = -(-m // 3), levels + 1
    return levels


def gpu_launches(stats, amg=0):
    """Kernel launches of the timed steps (counted from the solver statistics):
    per step 3 (stiffness) + 2 (BC) + 1 (preconditioner) + 2 (predictor);
    per Newton iteration 2 (force) + 1 (xyz update) + 1 (norm);
    per PCG iteration 3 with block-Jacobi, 4 + the V-cycle's 5 per level + 1
    with the multigrid preconditioner (amg = its levels; one sweep before and
    after each coarse correction); per reliable update 3 (block-Jacobi) or
    2 + the V-cycle."""
    per_it = 3 if not amg else 4 + 5 * amg + 1
    per_rel = 3 if not amg else 2 + 5 * amg + 1
    # multigrid, per step: the FP16 smoother copy (max, conversion), the FP64
    # copy for the true residual and the row sums of the difference form
    per_step = 8 if not amg else 12
    total = 0
    for st in stats:
        total += per_step + 4 * st["newton_iters"] + per_it * st["cg_iters"] + per_rel * st["refine_iters"] + \
            st["newton_iters"]
    return total


def run_e2e(args, case, precond, deadline):
    """The same steps through the reference-named C drop-in with the
    include/lpm.h globals on the host: the C host loop (liblpmhost.so, the
    src/lpmc_project.c:382-471 sequence) calls calcStiffness3DFiniteDifference,
    setDispBC, computeBondForceGeneral, updateRR, solverCG and switchStateV of
    liblpmgpu_legacy.so, which upload what each reads and write back what each
    writes.  Per-particle E as the reference expresses it: one type per
    particle with its own Ce row, boundary conditions by BC group."""
    try:
        import torch
        import lpm_gb300 as G
        import lpm_host
        os.environ["LPM_LEGACY_NO_KEXPORT"] = "1"
        h = lpm_host.HostDriver()
        n = h.setup(case.lattice, case.radius, case.box)
        s = G.Specimen(0)
        s.setup_lattice(case.lattice, case.radius, case.box)
        groups = cases.sc_types(h.get("xyz"), s.get("nb"), case.radius)
        s.close()
        h.set_types(np.arange(n, dtype=np.int32), n)
        h.set_bc_groups(groups, cases.NTYPE)
        c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
        u = cases.splitmix64_uniform(case.seed, n)
        sc = 1.0 + case.e_noise * (2.0 * u - 1.0)
        h.set_material(np.stack([c11 * sc, c12 * sc, c44 * sc], axis=1), 0, case.sigmay, 0.0, case.H)
        o = solver_opts(G, case, G.PREC_MIXED, precond)
        o.pop("newton_tol")
        o.pop("newton_maxiter")
        h.set_solver(**o)
        h.init()
        W, K = args.warmup, args.steps
        for k in range(W):
            h.load_step(cases.sc_bcs(case.schedule[k]), newton_tol=case.newton_tol, maxiter=100)
        h.traffic(reset=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(W, W + K):
            if deadline.left() < 0:
                return {"value": None, "unit": UNIT, "incomplete": f"deadline passed at step {k + 1}"}
            h.load_step(cases.sc_bcs(case.schedule[k]), newton_tol=case.newton_tol, maxiter=100)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        h2d, d2h = h.traffic()
        return {"value": K / dt, "unit": UNIT, "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "path": "C host loop (liblpmhost) -> reference-named drop-in (liblpmgpu_legacy), "
                        "include/lpm.h globals on the host",
                "material": "E +-5 % per particle: one type and Ce row per particle, BCs by BC group",
                "k_global_export": "off (LPM_LEGACY_NO_KEXPORT=1): the host copy of K_global is not read "
                                   "by the load-step loop; solverCG uses the device stiffness",
                "solver": "mixed precision, " + ("multigrid" if precond else "block-Jacobi") + " PCG"}
    except Exception as e:  # report, never fake
        return {"value": None, "unit": UNIT, "error": str(e)[:300]}


# Newton iterations per load step of the SC 100^3 cyclic case (E +-5 %,
# Newton tolerance 1e-8, MAXITER 100), steps 1-25, measured on a GB300 with
# FP64 multigrid-preconditioned solves to 1e-10; the count is the
# reference's modified-Newton iteration, independent of the linear solver at
# that solve accuracy (the per-step counts are summarised under profiles/).
NEWTON_PER_STEP_SC100 = [3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 8, 80, 88, 100, 100, 100, 100, 100, 100, 3, 3, 3, 3, 3]
# Block-Jacobi PCG iterations per Newton iteration at SC 100^3 (FP64, to
# 1e-8 relative, the tolerance of the reference's solverCG,
# src/solver.c:221, each solve from zero), measured on a GB300 over steps 4-8:
# 26,016 iterations in 15 solves (summarised under profiles/ with the
# per-step counts).
CG_PER_NEWTON_SC100 = 1734.4


def run_cpu_baseline(case, W, K):
    """Per-load-step cost of the reference algorithm at full size on the host
    cores (the oracle's C port of the reference path), from bounded samples
    of each phase, with the reference's own thread counts: the finite
    difference stiffness and the bond forces on nt_force = 3 threads
    (src/lpmc_project.c:57, :391, :452), the CG on all threads.  Per step:
    stiffness + Newton iterations x (force + CG iterations x one CG
    iteration), with the step's Newton count and the block-Jacobi PCG count
    per solve of the GPU runs (the reference's unpreconditioned CG needs at
    least as many)."""
    try:
        import oracle as O
        threads = os.cpu_count() or 1
        nt_force = min(3, threads)
        O.set_threads(threads)
        o = O.Oracle()
        t0 = time.perf_counter()
        n = o.setup_lattice(case.lattice, case.radius, case.box)
        setup_s = time.perf_counter() - t0
        types = cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius)
        o.set_types(types)
        u = cases.splitmix64_uniform(case.seed, n)
        sc = 1.0 + case.e_noise * (2.0 * u - 1.0)
        c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
        o.set_material(c11 * sc, c12 * sc, c44 * sc, case.sigmay, case.H, 0.0, 0)
        o.init_state()
        O.set_threads(nt_force)
        t0 = time.perf_counter()
        o.force(0)
        t_force = time.perf_counter() - t0
        O.set_threads(threads)
        nit = 10
        t0 = time.perf_counter()
        o.L.lo_cg_iterations(o.h, nit)
        t_cg = (time.perf_counter() - t0) / nit
        rows = min(n, 6000)
        t_fd = o.L.lo_fd_stiffness_timing(o.h, rows, nt_force) * n / rows  # last: it disturbs the state
        newton = NEWTON_PER_STEP_SC100[W:W + K] if case.n == 100 and W + K <= len(NEWTON_PER_STEP_SC100) \
            else [3] * K
        step_s = [t_fd + nn * (t_force + CG_PER_NEWTON_SC100 * t_cg) for nn in newton]
        total = sum(step_s)
        return {"value": K / total, "unit": UNIT, "cores": threads, "kind": "port",
                "ms_per_step": 1e3 * total / K,
                "sample": (f"oracle C port of the reference path at {n} particles: finite-difference stiffness "
                           f"of {rows} rows spread over the lattice on {nt_force} threads (scaled to all rows), "
                           f"one J2 force sweep on {nt_force} threads, {nit} CG iterations on the full upper "
                           f"CSR on {threads} threads; per step = stiffness + Newton iterations x (force + "
                           f"{CG_PER_NEWTON_SC100:.0f} CG iterations), Newton iterations of steps {W + 1}-{W + K} "
                           f"= {sum(newton)} (measured on the GPU, the same modified-Newton iteration)"),
                "threads": {"stiffness": nt_force, "force": nt_force, "cg": threads},
                "phase_s": {"fd_stiffness": t_fd, "force": t_force, "cg_iter": t_cg, "setup": setup_s}}
    except Exception as e:
        return {"value": None, "unit": UNIT, "kind": "port", "error": str(e)[:300]}


def run_batch(args):
    """Batched specimens: 256 SC specimens with independent edges U{20..60}
    (seed 1), per-specimen E ~ U[180, 220] GPa and yield ~ U[200, 400] MPa,
    H = 2 GPa, monotonic tension to 1% in 50 steps, all specimens in one batch
    context (one launch per kernel over all specimens, CUDA graphs per PCG
    chunk, launch shapes from the autotuner).  Compared with a loop of
    single-specimen solves of the same steps, timed on every 8th specimen and
    scaled by particle count."""
    import torch
    import lpm_gb300 as G
    torch.cuda.set_device(0)
    case = cases.BatchCase(nspec=args.nspec, seed=1)
    W, K = args.warmup, args.steps
    stream = torch.cuda.current_stream()
    prec = G.PREC_MIXED
    solver = dict(newton_maxiter=100, cg_rtol=1e-10, cg_maxiter=200000)
    t0 = time.perf_counter()
    s = G.Specimen(0)
    s.set_stream(stream.cuda_stream)
    n = s.setup_batch(case.lattice, case.radius, case.boxes)
    off = s.batch_offsets()
    xyz, nb = s.get("xyz"), s.get("nb")
    types = np.concatenate([cases.sc_types(xyz[off[k]:off[k + 1]], nb[off[k]:off[k + 1]], case.radius)
                            for k in range(case.nspec)])
    reps = np.diff(off)
    c11, c12, c44 = cases.iso_cubic(np.repeat(case.E, reps), case.nu)
    s.set_types(types)
    s.set_material(c11, c12, c44, np.repeat(case.sigmay, reps), np.full(n, case.H), 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=prec, newton_tol=case.newton_tol, **solver)
    setup_s = time.perf_counter() - t0
    bcs = case.step_bcs()
    tuning = None
    for k in range(W):
        s.batch_load_step(bcs)
        if k == 0:
            tuning = s.autotune()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stats = []
    for k in range(K):
        stats.append(s.batch_load_step(bcs))
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    ck = clocks.stop()
    du_batch = s.get("xyz") - s.get("xyz_initial")
    s.close()
    # loop of single-specimen solves on a sample of specimens
    sample = list(range(0, case.nspec, 8))
    loop_ms, err = 0.0, 0.0
    for k in sample:
        t = G.Specimen(0)
        t.set_stream(stream.cuda_stream)
        m = t.setup_lattice(case.lattice, case.radius, case.boxes[k])
        ty = cases.sc_types(t.get("xyz"), t.get("nb"), case.radius)
        a11, a12, a44 = cases.iso_cubic(case.E[k], case.nu)
        t.set_types(ty)
        t.set_material(np.full(m, a11), np.full(m, a12), np.full(m, a44), np.full(m, case.sigmay[k]),
                       np.full(m, case.H), 0.0, G.PL_J2)
        t.init_state()
        t.set_solver(precision=prec, newton_tol=case.newton_tol, **solver)
        for j in range(W):
            t.load_step(bcs[k])
            if j == 0:
                t.autotune()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for j in range(K):
            t.load_step(bcs[k])
        e1.record(stream)
        torch.cuda.synchronize()
        loop_ms += e0.elapsed_time(e1)
        d = t.get("xyz") - t.get("xyz_initial")
        ref = du_batch[off[k]:off[k + 1]]
        err = max(err, float(np.abs(d - ref).max() / np.abs(d).max()))
        t.close()
    share = float(sum(reps[k] for k in sample)) / float(n)
    loop_est_ms = loop_ms / share
    value = K / (ms / 1e3)
    agg = lambda key: int(sum(st[key] for step in stats for st in step))  # noqa: E731
    line = {
        "metric": "batch load steps/s, 256 SC specimens (edges U{20..60}), 1% tension",
        "value": value, "unit": "batch load steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 stiffness/SpMV/PCG + f64 residual, reliable updates and return map",
        "data": "synthetic (seeded specimen sizes and materials)",
        "config": {"workload": f"{case.nspec} SC specimens, edges U{{20..60}} seed 1, 1% tension in 50 steps, "
                               f"load steps {W + 1}-{W + K}",
                   "particles": n, "specimens": case.nspec, "setup_s": setup_s,
                   "specimen_steps_per_s": case.nspec * value,
                   "loop_of_single_solves_ms_per_step": loop_est_ms / K,
                   "batch_over_loop": loop_est_ms / ms,
                   "loop_sample": f"specimens {sample[0]}, {sample[1]}, ... every 8th ({len(sample)}), "
                                  f"{share:.3f} of the particles; loop time scaled by 1/share",
                   "max_rel_disp_diff_batch_vs_single": err,
                   "newton_iters": agg("newton_iters"), "cg_iters": agg("cg_iters"),
                   "reliable_updates": agg("refine_iters"), "tuning": tuning,
                   "l2": "inputs (15 GB of stiffness) far exceed the 129 MB L2"},
        "clocks": ck, "e2e": None, "cpu_baseline": None,
    }
    print(json.dumps(line))


def run_adjoint(args):
    """Differentiation workload: SC notched plate nx x 10 x nz (200 x 10 x 200:
    399,600 particles), single-edge notch 40 particles deep, smooth random
    per-particle E, nu, yield stress and H (Gaussian-filtered noise,
    correlation length 10 particles, +-10%, seed 1), 60 displacement steps to
    1% strain; loss = sum_n (R_n - R*_n)^2 with R* from the seed-2 fields.
    Times the forward run and the adjoint backward run (checkpoints every 10
    steps, recomputed), FP64, and checks one directional derivative per field
    against central differences (h = 1e-5 relative, two extra forward runs
    each) when --adj-fd is given."""
    import torch
    import lpm_gb300 as G
    torch.cuda.set_device(0)
    plate = cases.NotchedPlate(nx=args.plate_n, ny=10, nz=args.plate_n, notch=max(1, args.plate_n // 5),
                               steps=args.adj_steps, strain=args.adj_strain, corr=10.0)
    solver = dict(precision=G.PREC_FP64, newton_tol=args.adj_newton_tol, newton_maxiter=2000, cg_rtol=1e-12,
                  cg_maxiter=200000, newton_accel=8, cg_forcing=args.adj_forcing,
                  preconditioner=G.PRECOND_AMG if args.precond == "amg" else G.PRECOND_BJ)
    bcs = plate.step_bcs()

    def specimen():
        s = G.Specimen(0)
        s.setup_particles(plate.lattice, plate.radius, plate.xyz)
        s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), plate.radius))
        s.set_solver(**solver)
        return s

    f1, f2 = plate.fields(1), plate.fields(2)
    s = specimen()
    target = s.adjoint_forward(*f2, bcs, cases.T_TOP, "z")
    s.close()
    s = specimen()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    R = s.adjoint_forward(*f1, bcs, cases.T_TOP, "z", checkpoint_every=10)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    grads, st = s.adjoint_backward(2.0 * (R - target))
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    ck = clocks.stop()
    s.close()
    L = float(((R - target) ** 2).sum())
    fd = {}
    if args.adj_fd:
        names = ["E", "nu", "sigmay", "H"]
        for k in range(4):
            d = f1[k] * plate.fields(7 + k)[k] / plate.BASE[k]
            h = 1e-5
            Ls = []
            for sgn in (1.0, -1.0):
                f = [x.copy() for x in f1]
                f[k] = f1[k] + sgn * h * d
                t = specimen()
                Rp = t.adjoint_forward(*f, bcs, cases.T_TOP, "z")
                t.close()
                Ls.append(float(((Rp - target) ** 2).sum()))
            g_fd = (Ls[0] - Ls[1]) / (2 * h)
            g_ad = float((grads[names[k]] * d).sum())
            fd[names[k]] = {"adjoint": g_ad, "central_fd": g_fd, "rel_err": abs(g_fd - g_ad) / abs(g_ad)}
    line = {
        "metric": "adjoint gradient of a reaction-misfit loss: forward + backward seconds",
        "value": t2 - t0, "unit": "s", "n_gpus": 1, "steps": plate.steps, "warmup": 0,
        "higher_is_better": False, "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random fields)",
        "config": {"workload": f"SC notched plate {plate.nx}x{plate.ny}x{plate.nz}, notch {plate.notch}, "
                               f"{plate.steps} steps to {100 * plate.strain:g}% strain, loss vs seed-2 curve",
                   "particles": plate.n, "forward_s": t1 - t0, "backward_s": t2 - t1, "loss": L,
                   "adjoint_stats": st, "newton_tol": args.adj_newton_tol, "newton_accel": 8,
                   "cg_forcing": args.adj_forcing,
                   "checkpoint_every": 10, "fd_checks": fd},
        "clocks": ck, "e2e": None, "cpu_baseline": None,
    }
    print(json.dumps(line))


def run_fcc(args):
    """Crystal plasticity: FCC single crystal ncell^3 cells (80^3: 2,048,000
    particles), Al elastic constants, 24 signed {111}<110> systems, tau0 =
    50 MPa, linear hardening h0 = 500 MPa, [001] tension to 2% in 100 steps.
    Times load steps W+1..W+K on the mixed path and on the FP64 path and
    reports the displacement difference between them."""
    import torch
    import lpm_gb300 as G
    torch.cuda.set_device(0)
    case = cases.FCCCase(ncell=args.fcc_cells)
    W, K = args.fcc_warmup, args.steps
    stream = torch.cuda.current_stream()
    out = {}
    for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
        t0 = time.perf_counter()
        s = G.Specimen(0)
        s.set_stream(stream.cuda_stream)
        n = s.setup_lattice(case.lattice, case.radius, case.box)
        s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), case.radius))
        s.set_cp(*case.cp)
        s.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, G.PL_CP)
        s.init_state()
        # FP64 CG vectors with the FP32 stiffness: at 80^3 cells the FCC system
        # is too ill-conditioned for FP32 vectors (their PCG stagnates)
        amg = args.precond == "amg"
        s.set_solver(precision=prec, newton_tol=case.newton_tol, newton_maxiter=300, cg_rtol=1e-10,
                     cg_maxiter=2000 if amg else 40000, mixed_vectors=64,
                     preconditioner=G.PRECOND_AMG if amg else G.PRECOND_BJ, recycle=RECYCLE)
        setup_s = time.perf_counter() - t0
        warm = []
        for k in range(W):
            warm.append(s.load_step(cases.sc_bcs(case.schedule[k])))
            if k == 0:
                s.autotune()
        torch.cuda.synchronize()
        clocks = ClockSampler(0)
        clocks.start()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        stats = [s.load_step(cases.sc_bcs(case.schedule[k])) for k in range(W, W + K)]
        ev1.record(stream)
        torch.cuda.synchronize()
        out[name] = dict(ms=ev0.elapsed_time(ev1), stats=stats, warm=warm, clocks=clocks.stop(), n=n, setup_s=setup_s,
                         du=s.get("xyz") - s.get("xyz_initial"), A=s.get("cp_A"))
        s.close()
    m, f = out["mixed"], out["fp64"]
    value = K / (m["ms"] / 1e3)
    err = float(np.abs(m["du"] - f["du"]).max() / np.abs(f["du"]).max())
    agg = lambda st, key: int(sum(x[key] for x in st))  # noqa: E731
    line = {
        "metric": "load steps/s, FCC crystal plasticity, mixed vs FP64 GPU",
        "value": value, "unit": "load steps/s", "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": m["ms"] / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 stiffness and SpMV products, f64 PCG vectors, residual, reliable updates and CP return map",
        "data": "synthetic (FCC lattice)",
        "config": {"workload": f"FCC {args.fcc_cells}^3 cells CP [001] tension, load steps {W + 1}-{W + K} of 100",
                   "preconditioner": "smoothed-aggregation multigrid V-cycle" if args.precond == "amg"
                   else "block-Jacobi",
                   "particles": m["n"], "setup_s": m["setup_s"], "fp64_steps_per_s": K / (f["ms"] / 1e3),
                   "mixed_over_fp64": f["ms"] / m["ms"], "disp_err_mixed_vs_fp64": err,
                   "newton_iters": agg(m["stats"], "newton_iters"), "cg_iters": agg(m["stats"], "cg_iters"),
                   "fp64_newton_iters": agg(f["stats"], "newton_iters"), "fp64_cg_iters": agg(f["stats"], "cg_iters"),
                   "newton_iters_per_step": [st["newton_iters"] for st in m["stats"]],
                   "cg_iters_per_step": [st["cg_iters"] for st in m["stats"]],
                   "recycle": RECYCLE, "max_cp_A": float(m["A"].max()),
                   "fp64_fallbacks": agg(m["stats"], "fp64_fallbacks") + agg(m.get("warm", []), "fp64_fallbacks"),
                   "fp64_fallback_note": "mixed solves that failed with FP32 products and were redone with FP64 "
                                         "ones (the context keeps FP64 products from then on)"},
        "clocks": m["clocks"], "e2e": None, "cpu_baseline": None,
    }
    print(json.dumps(line))


def run_reference(args):
    """The reference arm: the reference's CPU algorithm (the oracle's C port,
    bit-identical to the reference on every pinned case) on the host cores,
    on this arm's workload, metric and unit.  Under torchrun only rank 0
    measures; the other ranks exit without work."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    case = cases.SCCase(n=args.size, e_noise=0.05, seed=1)
    cpu = run_cpu_baseline(case, args.warmup, args.steps)
    v = cpu.get("value")
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": cpu.get("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded lattice and per-particle material noise)",
            "config": {"workload": f"SC {args.size}^3 elastoplastic cyclic (E +-5 % per particle), load steps "
                                   f"{args.warmup + 1}-{args.warmup + args.steps}"},
            "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=100)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--arm-precision", default="mixed", choices=["mixed", "fp64"],
                    help="precision of the first (headline) arm; fp64 with --no-fp64 profiles the comparator "
                         "alone")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--workload", default="sc", choices=["sc", "batch", "adjoint", "fcc"],
                    help="sc: the 1M-particle SC cyclic case (default); batch: 256 specimens; "
                         "adjoint: gradients on the notched plate; fcc: crystal plasticity")
    ap.add_argument("--fcc-cells", type=int, default=80)
    ap.add_argument("--fcc-warmup", type=int, default=7,
                    help="warm-up load steps of the fcc workload (at 80^3 cells the crystal first slips in "
                         "step 8; time it with --steps 1)")
    ap.add_argument("--adj-strain", type=float, default=0.01)
    ap.add_argument("--nspec", type=int, default=256)
    ap.add_argument("--plate-n", type=int, default=200)
    ap.add_argument("--adj-steps", type=int, default=60)
    ap.add_argument("--adj-newton-tol", type=float, default=1e-10)
    ap.add_argument("--adj-forcing", type=float, default=0.0,
                    help="adjoint workload: inexact-Newton forcing cap (opts.cg_forcing; 0 = exact solves)")
    ap.add_argument("--adj-fd", action="store_true")
    ap.add_argument("--precond", default="amg", choices=["bj", "amg"],
                    help="sc, fcc and adjoint workloads: PCG preconditioner (the multigrid V-cycle or "
                         "block-Jacobi)")
    ap.add_argument("--budget", type=float, default=1450.0,
                    help="sc workload: wall seconds from start within which the arms must fit")
    ap.add_argument("--grace", type=float, default=200.0,
                    help="sc workload: the watchdog prints the line measured so far at budget + grace")
    ap.add_argument("--cg-rtol", type=float, default=CG_RTOL,
                    help="sc workload: relative residual of the linear solves (the reference's solverCG "
                         "stops at 1e-8, src/solver.c:221)")
    ap.add_argument("--diff-stream", type=int, default=DIFF_STREAM, choices=[-1, 0, 1, 2, 3],
                    help="sc workload, mixed multigrid: difference-form product fed by registers (0) or streamed "
                         "through shared memory (1, 2: tiles of 16 rows, 1 or 2 thread blocks per SM; 3: tiles of "
                         "8 rows, 5 per SM); -1 keeps the autotuner's choice")
    ap.add_argument("--smooth-stream", type=int, default=SMOOTH_STREAM, choices=[-1, 0, 1, 2, 3],
                    help="sc workload, multigrid: level-0 smoother fed by registers (0) or streamed through shared "
                         "memory (as --diff-stream; 3: 6 thread blocks per SM); -1 keeps the autotuner's choice")
    ap.add_argument("--recycle", type=int, default=RECYCLE,
                    help="earlier solutions of the load step each Newton solve starts from (0: from zero, "
                         "as the reference's solverCG)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    globals()["CG_RTOL"] = args.cg_rtol
    globals()["RECYCLE"] = args.recycle
    globals()["DIFF_STREAM"] = args.diff_stream
    globals()["SMOOTH_STREAM"] = args.smooth_stream
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "fcc":
        run_fcc(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

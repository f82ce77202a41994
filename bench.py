"""Benchmark: load steps/s of the 1M-particle SC elastoplastic cyclic case.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one load step of src/lpmc_project.c:385-471): simple
cubic lattice 100 x 100 x 100 (1e6 particles, 8.9e6 bonds, 3e6 DOF),
spacing 0.2 mm, E = 200 GPa with +-5% uniform noise per particle (seed 1),
nu = 0.3, J2 yield 250 MPa, linear hardening 2 GPa; bottom face fixed in z
(plus a 3-DOF rigid-body pin), top face displaced along the +-0.2% strain
cycle, 20 steps per quarter cycle; Newton tolerance 1e-8, block-Jacobi PCG
to relative residual 1e-10.  The W warm-up steps are the first W steps of
the schedule; the K timed steps follow them.

Headline: the mixed-precision path (FP32 stiffness/SpMV/PCG with FP64
reliable updates, FP64 residuals and return map).  The same steps run on the
plain FP64 path for the ratio and the displacement error between the two.
Inputs are resident in HBM (value); `e2e` runs the same steps through the
reference-named C drop-in (liblpmhost.so + liblpmgpu_legacy.so) with the
include/lpm.h globals on the host, host<->device copies inside the timed
region.  The reference arm times the oracle's C port of the reference
algorithm on the host cores.
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
    # the multigrid PCG needs about 25 iterations per solve: a low cap bounds
    # the time a misbehaving solve can take
    s.set_solver(precision=precision, newton_tol=case.newton_tol, newton_maxiter=100, cg_rtol=1e-10,
                 cg_maxiter=2000 if precond else 200000, preconditioner=precond)
    return s, types


def run_ours(args):
    import torch
    import lpm_gb300 as G
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    case = cases.SCCase(n=args.size, e_noise=0.05, seed=1)
    sched = case.schedule
    W, K = args.warmup, args.steps
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    results = {}
    for prec_name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
        if prec_name == "fp64" and args.no_fp64:
            continue
        precond = G.PRECOND_AMG if args.precond == "amg" else G.PRECOND_BJ
        s, types = build_specimen(G, case, prec, stream.cuda_stream, precond)
        tuning = None
        warm = []
        for k in range(W):
            warm.append(s.load_step(cases.sc_bcs(sched[k])))
            if k == 0 and not args.no_autotune:
                tuning = s.autotune()  # launch shapes from the project's autotuner
        barrier()
        s.spmv_timing(reset=2)
        clocks = ClockSampler(local)
        clocks.start()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stats = []
        barrier()
        ev0.record(stream)
        for k in range(W, W + K):
            stats.append(s.load_step(cases.sc_bcs(sched[k])))
        ev1.record(stream)
        barrier()
        ms = ev0.elapsed_time(ev1)
        ck = clocks.stop()
        spmv_ms, spmv_cnt = s.spmv_timing(reset=3)
        ms = max_over_ranks(ms, device="cuda")
        results[prec_name] = dict(ms=ms, stats=stats, warm=warm, spmv_ms=spmv_ms, spmv_cnt=spmv_cnt, clocks=ck,
                                  tuning=tuning,
                                  spmv_bytes=s.spmv_bytes(prec), xyz=s.get("xyz"), x0=s.get("xyz_initial"),
                                  n=s.n, nnzb=s.sizes()["nnz_blocks"])
        s.close()
        del s
    mixed = results["mixed"]
    value = world * K / (mixed["ms"] / 1e3)
    hbm, peak_src = peaks()
    achieved = mixed["spmv_bytes"] / (mixed["spmv_ms"] * 1e-3) / 1e9 if mixed["spmv_ms"] > 0 else None
    traffic = spmv_traffic(mixed["spmv_bytes"])
    err = None
    fp64_rate = None
    if "fp64" in results:
        f = results["fp64"]
        fp64_rate = world * K / (f["ms"] / 1e3)
        du_m = mixed["xyz"] - mixed["x0"]
        du_f = f["xyz"] - f["x0"]
        err = float(np.abs(du_m - du_f).max() / np.abs(du_f).max())
    if args.compare_du:
        ref = np.load(args.compare_du)
        du = mixed["xyz"] - mixed["x0"]
        err = float(np.abs(du - ref).max() / np.abs(ref).max())
    e2e = run_e2e(args, case) if (not args.no_e2e and rank == 0) else None
    counts = step_counts(args.size, W, K, results["fp64"]["stats"] if "fp64" in results else None)
    cpu = run_cpu_baseline(args, case, counts) if (not args.no_cpu and rank == 0) else None
    agg = lambda key: int(sum(st[key] for st in mixed["stats"]))  # noqa: E731
    amg = None
    if args.precond == "bj" and not args.no_amg and world == 1:
        amg = run_amg_side(args, mixed["xyz"] - mixed["x0"], value)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": mixed["ms"] / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 stiffness/SpMV/PCG + f64 residual, refinement and return map",
        "data": "synthetic (seeded lattice and material noise)",
        "config": {"workload": f"SC {args.size}^3 elastoplastic cyclic, load steps {W + 1}-{W + K} of "
                               f"{len(sched)} (first yield near step 12)",
                   "particles": mixed["n"], "nnz_blocks": mixed["nnzb"], "precision": "mixed",
                   "preconditioner": "smoothed-aggregation multigrid V-cycle" if args.precond == "amg"
                   else "block-Jacobi",
                   "fp64_steps_per_s": fp64_rate, "mixed_over_fp64": (value / fp64_rate) if fp64_rate else None,
                   "disp_err_mixed_vs_fp64": err, "newton_iters": agg("newton_iters"), "cg_iters": agg("cg_iters"),
                   "reliable_updates": agg("refine_iters"),
                   "fp64_cg_iters": (sum(st["cg_iters"] for st in results["fp64"]["stats"])
                                     if "fp64" in results else None),
                   "l2": "SpMV stream of 2.4 GB per call > 129 MB L2 (no flush needed)",
                   "tuning": mixed["tuning"],
                   "amg_build_ms": sum(st["ms_amg_build"] for st in mixed["warm"] + mixed["stats"]),
                   "amg_builds": sum(st["amg_builds"] for st in mixed["warm"] + mixed["stats"]),
                   "multigrid": amg,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                     "kernel": "k_spmv_f (FP32 block-CSR SpMV)", "peak_source": peak_src,
                     "spmv_launches_sampled": mixed["spmv_cnt"]},
        "clocks": mixed["clocks"],
        "gpu_launches": gpu_launches(mixed["stats"], amg_levels(mixed["n"]) if args.precond == "amg" else 0),
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_amg_side(args, du_bj, bj_value):
    """The same workload with the multigrid preconditioner, measured in a child
    process after the block-Jacobi line is complete (a failure there cannot
    cost the headline): its load steps/s, the ratio to block-Jacobi, PCG
    iterations, hierarchy build time, and its displacements against
    block-Jacobi's."""
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        ref = os.path.join(d, "du_bj.npy")
        np.save(ref, du_bj)
        cmd = [sys.executable, os.path.abspath(__file__), "--precond", "amg", "--no-fp64", "--no-e2e", "--no-cpu",
               "--no-amg", "--steps", str(args.steps), "--warmup", str(args.warmup), "--size", str(args.size),
               "--compare-du", ref]
        if args.no_autotune:
            cmd.append("--no-autotune")
        try:
            out = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
        except subprocess.TimeoutExpired:
            return {"error": "timed out after 300 s"}
        lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
        if out.returncode != 0 or not lines:
            tail = (out.stderr or out.stdout).strip().splitlines()[-1:] or [""]
            return {"error": f"exit {out.returncode}: {tail[0][:300]}"}
        line = json.loads(lines[-1])
    c = line["config"]
    return {"steps_per_s": line["value"], "ms_per_step": line["ms_per_step"],
            "over_block_jacobi": line["value"] / bj_value if bj_value else None,
            "cg_iters": c["cg_iters"], "newton_iters": c["newton_iters"], "reliable_updates": c["reliable_updates"],
            "hierarchy_builds": c["amg_builds"], "hierarchy_build_ms": c["amg_build_ms"],
            "disp_err_vs_block_jacobi": c["disp_err_mixed_vs_fp64"], "gpu_launches": line["gpu_launches"],
            "clocks": line.get("clocks")}


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
    total = 0
    for st in stats:
        total += 8 + 4 * st["newton_iters"] + per_it * st["cg_iters"] + per_rel * st["refine_iters"] + \
            st["newton_iters"]
    return total


def run_e2e(args, case):
    """Same steps through the reference-named C drop-in with host globals."""
    try:
        import torch
        import lpm_gb300 as G
        import lpm_host
        h = lpm_host.HostDriver()
        n = h.setup(case.lattice, case.radius, case.box)
        # particle types as for the GPU specimen (the legacy ABI selects BCs by
        # type and takes Ce per type, so this leg runs with uniform E)
        s = G.Specimen(0)
        s.setup_lattice(case.lattice, case.radius, case.box)
        types = cases.sc_types(h.get("xyz"), s.get("nb"), case.radius)
        s.close()
        h.set_types(types, cases.NTYPE)
        h.set_material(np.tile(cases.iso_cubic(case.E, case.nu), (cases.NTYPE, 1)), 0, case.sigmay, 0.0, case.H)
        h.set_solver(precision=G.PREC_MIXED, cg_rtol=1e-10, cg_maxiter=200000)
        h.init()
        W, K = args.warmup, args.steps
        for k in range(W):
            h.load_step(cases.sc_bcs(case.schedule[k]), newton_tol=case.newton_tol)
        h.traffic(reset=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(W, W + K):
            h.load_step(cases.sc_bcs(case.schedule[k]), newton_tol=case.newton_tol)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        h2d, d2h = h.traffic()
        return {"value": K / dt, "unit": UNIT, "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "path": "C host loop (liblpmhost) -> reference-named drop-in (liblpmgpu_legacy), "
                        "include/lpm.h globals on the host",
                "note": "uniform E (per-particle E needs one Ce row per particle in the legacy ABI)"}
    except Exception as e:  # report, never fake
        return {"value": None, "unit": UNIT, "error": str(e)[:300]}


COUNTS_FILE = os.path.join(ROOT, "profiles", "iteration_counts_sc100.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "k_spmv_f_traffic.json")


def spmv_traffic(alg_bytes):
    """DRAM bytes (read + write) per SpMV launch: the ncu capture of a smaller
    case (dram__bytes_read.sum + dram__bytes_write.sum) scaled to this launch
    by its algorithmic bytes, which grow with the block count."""
    try:
        with open(TRAFFIC_FILE) as f:
            d = json.load(f)
        return alg_bytes * d["traffic_over_algorithmic"]
    except Exception:
        return None


def step_counts(size, W, K, stats=None):
    """Newton iterations per step and CG iterations per Newton iteration of the
    timed steps: from this run when available, else from the committed record
    of an earlier FP64 GPU run of the same steps, else a model."""
    if stats:
        newton = sum(st["newton_iters"] for st in stats) / len(stats)
        cg = sum(st["cg_iters"] for st in stats) / max(1.0, sum(st["newton_iters"] for st in stats))
        return newton, cg, "this run's FP64 GPU counts"
    try:
        with open(COUNTS_FILE) as f:
            d = json.load(f)
        # per-step averages over the recorded steps (the elastic steps 4-8
        # all take 3 Newton iterations), valid for timed runs starting there
        if d.get("size") == size and d.get("first_step") == W + 1:
            return d["newton_per_step"], d["cg_per_newton"], "recorded FP64 GPU counts (" + COUNTS_FILE[len(ROOT) + 1:] + ")"
    except Exception:
        pass
    return 2.0, 1800.0, "model: 2 Newton iterations, 1800 CG iterations each"


def run_cpu_baseline(args, case, counts):
    """Per-load-step cost of the reference algorithm (the oracle's C port, all
    host threads) at full size, from bounded samples of each phase."""
    try:
        import oracle as O
        threads = os.cpu_count() or 1
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
        rows = min(n, 2000)
        r0 = min(n // 2, n - rows)  # a sample of interior rows that fits the lattice
        t0 = time.perf_counter()
        o.L.lo_fd_stiffness_range(o.h, r0, r0 + rows)  # serial, as the reference's side effects require
        t_fd = (time.perf_counter() - t0) * n / rows / threads  # the reference runs it OpenMP-parallel
        t0 = time.perf_counter()
        o.force(0)
        t_force = time.perf_counter() - t0
        nit = 10
        t0 = time.perf_counter()
        o.L.lo_cg_iterations(o.h, nit)
        t_cg = (time.perf_counter() - t0) / nit
        newton, cgit, src = counts
        step_s = t_fd + newton * (t_force + cgit * t_cg)
        return {"value": 1.0 / step_s, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": (f"oracle C port of the reference path at {n} particles: FD stiffness of {rows} "
                           f"rows (scaled to all rows and {threads} threads), one J2 force sweep, {nit} "
                           f"threaded CG iterations on the full upper CSR; per step = FD + {newton:.1f} "
                           f"Newton x (force + {cgit:.0f} CG iterations) - counts: {src} (the reference's "
                           f"unpreconditioned CG needs more, so this flatters the CPU)"),
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
        s.set_solver(precision=prec, newton_tol=case.newton_tol, newton_maxiter=300, cg_rtol=1e-10,
                     cg_maxiter=40000, mixed_vectors=64,
                     preconditioner=G.PRECOND_AMG if args.precond == "amg" else G.PRECOND_BJ)
        setup_s = time.perf_counter() - t0
        for k in range(W):
            s.load_step(cases.sc_bcs(case.schedule[k]))
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
        out[name] = dict(ms=ev0.elapsed_time(ev1), stats=stats, clocks=clocks.stop(), n=n, setup_s=setup_s,
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
                   "max_cp_A": float(m["A"].max())},
        "clocks": m["clocks"], "e2e": None, "cpu_baseline": None,
    }
    print(json.dumps(line))


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    case = cases.SCCase(n=args.size, e_noise=0.05, seed=1)
    cpu = run_cpu_baseline(args, case, step_counts(args.size, args.warmup, args.steps))
    line = {"metric": METRIC, "impl": "reference", "value": cpu.get("value"), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "vs_baseline": None,
            "config": {"workload": f"SC {args.size}^3 elastoplastic cyclic"},
            "cpu_baseline": cpu,
            "e2e": {"value": cpu.get("value"), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=100)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--workload", default="sc", choices=["sc", "batch", "adjoint", "fcc"],
                    help="sc: the 1M-particle SC cyclic case (default); batch: 256 specimens; "
                         "adjoint: gradients on the notched plate; fcc: crystal plasticity")
    ap.add_argument("--fcc-cells", type=int, default=80)
    ap.add_argument("--fcc-warmup", type=int, default=1,
                    help="warm-up load steps of the fcc workload (its steps are long)")
    ap.add_argument("--adj-strain", type=float, default=0.01)
    ap.add_argument("--nspec", type=int, default=256)
    ap.add_argument("--plate-n", type=int, default=200)
    ap.add_argument("--adj-steps", type=int, default=60)
    ap.add_argument("--adj-newton-tol", type=float, default=1e-10)
    ap.add_argument("--adj-forcing", type=float, default=0.0,
                    help="adjoint workload: inexact-Newton forcing cap (opts.cg_forcing; 0 = exact solves)")
    ap.add_argument("--adj-fd", action="store_true")
    ap.add_argument("--precond", default="bj", choices=["bj", "amg"],
                    help="sc, fcc and adjoint workloads: PCG preconditioner (block-Jacobi or the multigrid V-cycle)")
    ap.add_argument("--no-amg", action="store_true",
                    help="sc workload: skip the side measurement with the multigrid preconditioner")
    ap.add_argument("--compare-du", default=None, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
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

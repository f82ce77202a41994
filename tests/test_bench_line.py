"""bench.py's JSON line on the CPU: the line is assembled from whatever arms
finished (a skipped or unfinished arm leaves its fields null with the
reason), and the reference arm prints a complete line for a small lattice."""
import json
import os
import subprocess
import sys
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
import cases  # noqa: E402


def _args(**kw):
    a = dict(steps=2, warmup=3, size=10, precond="amg", no_autotune=False)
    a.update(kw)
    return SimpleNamespace(**a)


def _stat(newton, cg):
    return {"newton_iters": newton, "cg_iters": cg, "refine_iters": 2, "amg_builds": 0, "ms_amg_build": 0.0}


def _arm(ms, du_scale=1.0):
    x0 = np.zeros((8, 3))
    return dict(ms=ms, stats=[_stat(3, 90), _stat(80, 3000)], warm=[_stat(3, 90)] * 3, spmv_ms=0.5, spmv_cnt=10,
                clocks={"sm_mhz": 1900.0}, tuning=None, spmv_bytes=2.4e9, xyz=x0 + du_scale, x0=x0,
                alpha=np.full(8, 1e-3 * du_scale), react=100.0 * du_scale, n=8, nnzb=64, setup_s=1.0,
                step_wall_s=[0.5, 20.0])


def test_line_complete():
    c = cases.SCCase(n=10)
    line = bench.assemble_line(_args(), c, {"mixed": _arm(1000.0), "fp64": _arm(2000.0, 1.0 + 1e-9),
                                            "e2e": {"value": 1.0}, "cpu": {"value": 0.01}}, 1)
    assert line["value"] == 2.0 and line["ms_per_step"] == 500.0
    cfg = line["config"]
    assert cfg["mixed_over_fp64"] == 2.0 and cfg["fp64_steps_per_s"] == 1.0
    assert 0.0 < cfg["disp_err_mixed_vs_fp64"] < 2e-9
    assert cfg["newton_iters_per_step"] == [3, 80] and cfg["newton_iters"] == 83
    rl = line["roofline"]
    assert abs(rl["achieved"] - 2.4e9 / 0.5e-3 / 1e9) < 1e-6 and rl["frac"] == rl["achieved"] / rl["peak"]
    assert line["e2e"]["value"] == 1.0 and line["cpu_baseline"]["value"] == 0.01
    assert line["gpu_launches"] > 0
    json.dumps(line)


def test_line_names_the_streamed_product():
    """With the autotuner's streamed product the roofline names that kernel
    and scales its own measured traffic ratio."""
    c = cases.SCCase(n=10)
    mixed = _arm(1000.0)
    mixed["tuning"] = {"diff_stream": 3, "smooth_stream": 3}
    line = bench.assemble_line(_args(), c, {"mixed": mixed, "fp64": _arm(2000.0), "e2e": None, "cpu": None}, 1)
    rl = line["roofline"]
    assert rl["kernel"].startswith("k_spmv_diff_stream")
    assert abs(rl["traffic"] - 2.4e9 * bench.SPMV_STREAM_TRAFFIC_OVER_ALG) < 1.0
    line = bench.assemble_line(_args(), c, {"mixed": _arm(1000.0), "fp64": _arm(2000.0), "e2e": None, "cpu": None},
                               1)
    assert line["roofline"]["kernel"].startswith("k_spmv_diff (")
    assert abs(line["roofline"]["traffic"] - 2.4e9 * bench.SPMV_TRAFFIC_OVER_ALG) < 1.0


def test_line_with_skipped_arms():
    c = cases.SCCase(n=10)
    line = bench.assemble_line(_args(), c, {"mixed": _arm(1000.0), "fp64": {"skipped": "budget: 10 s left"},
                                            "e2e": {"value": None, "skipped": "budget"}, "cpu": None}, 1)
    assert line["value"] == 2.0
    cfg = line["config"]
    assert cfg["fp64_steps_per_s"] is None and cfg["mixed_over_fp64"] is None
    assert cfg["fp64_arm"] == {"skipped": "budget: 10 s left"}
    json.dumps(line)


def test_line_when_headline_unfinished():
    c = cases.SCCase(n=10)
    line = bench.assemble_line(_args(), c, {"mixed": {"incomplete": "deadline passed before timed step 9"}}, 1,
                               note="hard time limit reached")
    assert line["value"] is None and line["ms_per_step"] is None and line["roofline"]["achieved"] is None
    assert line["config"]["mixed_arm"]["incomplete"].startswith("deadline")
    assert line["config"]["note"] == "hard time limit reached"
    json.dumps(line)


def test_reference_arm_small_lattice():
    """The reference arm (the oracle's C port timed on the host) prints its
    JSON line for a lattice smaller than its stiffness sample."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--size", "8"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0.0 and line["ms_per_step"] > 0.0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["threads"]["stiffness"] <= 3

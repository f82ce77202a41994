"""bench.py's multigrid side measurement on the CPU: the child run's JSON line
becomes the `multigrid` entry of the headline's config, and a failing child
becomes an error entry instead of failing the headline."""
import json
import os
import subprocess
import sys
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _args():
    return SimpleNamespace(steps=5, warmup=3, size=100, no_autotune=False)


def test_side_run_parsed(monkeypatch):
    line = {"value": 1.0, "ms_per_step": 1000.0, "gpu_launches": 123, "clocks": {"sm_mhz": 1900},
            "config": {"cg_iters": 500, "newton_iters": 25, "reliable_updates": 40, "amg_builds": 1,
                       "amg_build_ms": 9000.0, "disp_err_mixed_vs_fp64": 2e-11}}
    seen = {}

    def fake_run(cmd, **kw):
        seen["cmd"] = cmd
        ref = cmd[cmd.index("--compare-du") + 1]
        assert np.load(ref).shape == (8, 3)
        return SimpleNamespace(returncode=0, stdout="warm-up noise\n" + json.dumps(line) + "\n", stderr="")
    monkeypatch.setattr(subprocess, "run", fake_run)
    out = bench.run_amg_side(_args(), np.ones((8, 3)), 0.2)
    assert out["steps_per_s"] == 1.0 and abs(out["over_block_jacobi"] - 5.0) < 1e-12
    assert out["cg_iters"] == 500 and out["hierarchy_build_ms"] == 9000.0
    assert out["disp_err_vs_block_jacobi"] == 2e-11
    cmd = seen["cmd"]
    assert cmd[cmd.index("--precond") + 1] == "amg" and "--no-amg" in cmd and "--no-cpu" in cmd


def test_side_run_failure_is_reported(monkeypatch):
    monkeypatch.setattr(subprocess, "run",
                        lambda cmd, **kw: SimpleNamespace(returncode=1, stdout="", stderr="Traceback\nLPMError: x\n"))
    out = bench.run_amg_side(_args(), np.ones((8, 3)), 0.2)
    assert out == {"error": "exit 1: LPMError: x"}

    def timeout(cmd, **kw):
        raise subprocess.TimeoutExpired(cmd, 300)
    monkeypatch.setattr(subprocess, "run", timeout)
    assert "timed out" in bench.run_amg_side(_args(), np.ones((8, 3)), 0.2)["error"]


def test_reference_arm_small_lattice():
    """The reference arm (the oracle's C port timed on the host) prints its
    JSON line for a lattice smaller than its FD-stiffness sample."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--size", "8"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0.0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0

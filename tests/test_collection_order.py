"""GPU tests marked gpu_last are collected after every other GPU test, so a
failure among the not-yet-run cases cannot stop a fail-fast GPU run early."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_gpu_last_tests_come_last():
    out = subprocess.run([sys.executable, "-m", "pytest", "tests", "-m", "gpu", "--collect-only", "-q"],
                         capture_output=True, text=True, cwd=ROOT, timeout=300)
    ids = [l for l in out.stdout.splitlines() if "::" in l]
    assert ids, out.stdout[-2000:]
    late = {"test_gpu_amg.py", "test_gpu_forcing.py", "test_gpu_kinematic.py"}
    first_late = next(k for k, t in enumerate(ids) if t.split("::")[0].split("/")[-1] in late)
    tail = ids[first_late:]
    # everything after the first late test is late too
    assert all(t.split("::")[0].split("/")[-1] in late or "match_oracle" in t or "bit_exact" in t or "vs_fd" in t
               for t in tail), tail
    assert any("test_load_steps_match_oracle" in t for t in ids[:first_late])
    assert any("test_force_bc_steps_match_oracle" in t for t in tail)

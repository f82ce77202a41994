"""GPU collection order: the established tests, then the later
reference-pinned parity cases (gpu_last), then the opt-in solver options
(gpu_option: multigrid, inexact and accelerated Newton), then the
allocation-free entry point's file, so that a fail-fast run reaches every
parity test before an optional feature can stop it."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OPTION_FILES = {"test_gpu_amg.py", "test_gpu_forcing.py", "test_gpu_anderson.py", "test_gpu_recycle.py",
                "test_gpu_stream.py"}


def _fname(t):
    return t.split("::")[0].split("/")[-1]


def test_gpu_collection_tiers():
    out = subprocess.run([sys.executable, "-m", "pytest", "tests", "-m", "gpu", "--collect-only", "-q"],
                         capture_output=True, text=True, cwd=ROOT, timeout=300)
    ids = [l for l in out.stdout.splitlines() if "::" in l]
    assert ids, out.stdout[-2000:]
    files = [_fname(t) for t in ids]
    # the allocation-free entry point's tests come last of all
    first_zz = next(k for k, f in enumerate(files) if f.startswith("test_zz_"))
    assert all(f.startswith("test_zz_") for f in files[first_zz:])
    # the solver options come right before them, after every parity case
    first_opt = next(k for k, f in enumerate(files) if f in OPTION_FILES)
    assert all(f in OPTION_FILES for f in files[first_opt:first_zz])
    assert not any(f in OPTION_FILES for f in files[:first_opt])
    head = ids[:first_opt]
    for name in ("test_load_steps_match_oracle", "test_force_bc_steps_match_oracle",
                 "test_per_particle_moduli_match_oracle", "test_kinematic"):
        assert any(name in t for t in head), name

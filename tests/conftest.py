import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "lpm-c_gb300"),
          os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "gpu_last: reference-pinned GPU parity cases collected after the "
                                       "established ones")
    config.addinivalue_line("markers", "gpu_option: GPU tests of opt-in solver options (multigrid, inexact "
                                       "and accelerated Newton); collected after every parity test, so "
                                       "that a failure there cannot stop a fail-fast run before them")


def _tier(item):
    """Collection tier: established tests, then the later reference-pinned
    parity cases, then the opt-in solver options, then the allocation-free
    entry point's file (test_zz_*), which always comes last."""
    if item.fspath.basename.startswith("test_zz_"):
        return 3
    if item.get_closest_marker("gpu_option"):
        return 2
    if item.get_closest_marker("gpu_last"):
        return 1
    return 0


def pytest_collection_modifyitems(config, items):
    items.sort(key=_tier)  # stable: file order within a tier


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    import lpm_gb300
    lpm_gb300.load()
    return lpm_gb300


def golden(name):
    import numpy as np
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip(f"golden fixture {name} missing")
    return np.load(path)

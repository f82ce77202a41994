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
    config.addinivalue_line("markers", "gpu_last: GPU cases that have not run on a GPU yet; collected after "
                                       "the others, so that a failure among them cannot stop a fail-fast "
                                       "run before the established tests")


def pytest_collection_modifyitems(config, items):
    late = [i for i in items if i.get_closest_marker("gpu_last")]
    if late:
        items[:] = [i for i in items if not i.get_closest_marker("gpu_last")] + late


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

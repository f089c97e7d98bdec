"""Shared pytest configuration: the `gpu` marker and paths."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


@pytest.fixture(scope="session", autouse=True)
def _native_library():
    """The library (host planner and kernels) built in-tree before any test: nvcc cross-compiles
    it without a GPU, and the build is skipped when it is up to date."""
    from tnkit_gb300 import build
    build.build()


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    with open(os.path.join(GOLDEN, "local_problems.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, "local_problems.npz")))
    return meta, arrays

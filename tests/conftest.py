import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and libmplicits.so")


def pytest_collection_modifyitems(config, items):
    import torch
    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def tiny_levels():
    """The three 3->32->32->32->1 levels of tests/golden/tiny_three_level.npz
    as oracle parameter lists and as state_dicts."""
    d = golden("tiny_three_level.npz")
    levels, sds = [], []
    for i in range(3):
        sd = {}
        for j in range(4):
            sd[f"net.{j}.0.weight"] = d[f"L{i}.net.{j}.0.weight"]
            sd[f"net.{j}.0.bias"] = d[f"L{i}.net.{j}.0.bias"]
        params = [(sd[f"net.{j}.0.weight"], sd[f"net.{j}.0.bias"]) for j in range(4)]
        levels.append((params, [30.0, 30.0, 30.0]))
        sds.append(sd)
    return levels, sds, d


@pytest.fixture(scope="session")
def lib():
    from mplicits_gb300 import build, capi
    build.build()
    return capi.load()

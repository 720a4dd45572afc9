"""Shared test configuration.

Tests marked ``gpu`` need a CUDA GPU and the built ``libdompap_gpu.so``; all
other tests run on the CPU (the oracle against the golden fixtures, host
logic, and that the C ABI library loads and exports its symbols).
"""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: long-running test")


def load_golden(name):
    data = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    return {k: data[k] for k in data.files}


@pytest.fixture(scope="session")
def golden_unit():
    return load_golden("golden_unit.npz")


@pytest.fixture(scope="session")
def golden_configs():
    return load_golden("golden_configs.npz")


@pytest.fixture(scope="session")
def golden_traj():
    return load_golden("golden_traj.npz")


CONFIG_TAGS = ["lj500", "harm3d", "harm2d", "harm4d", "hard3d", "sig2eps4", "wahn", "callable", "expensive"]


def config_of(golden, tag):
    return {k.split("/", 1)[1]: v for k, v in golden.items() if k.startswith(tag + "/")}

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "modal-cmb_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libmodal_gb300.so")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build_oracle()
    return oracle.Oracle()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name + ".npz"))
    return load


@pytest.fixture(scope="session")
def mg():
    import modal_gb300
    return modal_gb300


def rel_fro(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

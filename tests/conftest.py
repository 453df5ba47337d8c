import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and runs the drop-in library on it")


@pytest.fixture(scope="session")
def gpu_lib():
    from peeeeeeeeeeeeeeeeeeec_gb300 import abi
    lib = abi.load_gpu_lib()
    if not lib.peec_gb300_device_ready():
        raise RuntimeError("CUDA device not available to libpeec_gb300.so")
    return lib


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name + ".npz"))

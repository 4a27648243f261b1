import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def pk():
    from exshalos_gb300.workloads import synthetic_pk
    k, P = synthetic_pk()
    return k.astype(np.float32), P.astype(np.float32)


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as o
    o.lib("f64")
    o.lib("f32")
    return o


def rel_rms(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2) / np.mean(b ** 2)))

"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else
runs on the CPU (oracle, host plan logic, C ABI loading)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def uniform_cloud(n, d, seed=0):
    """n points i.i.d. uniform in [0,1]^d, dim x n (numpy default_rng(seed))."""
    return np.random.default_rng(seed).random((d, n))


def sphere_cloud(n, seed=0):
    """n points on S^2 from normalised N(0, I_3) draws."""
    P = np.random.default_rng(seed).standard_normal((3, n))
    return P / np.linalg.norm(P, axis=0)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)

"""Shared fixtures; registers the ``gpu`` marker (tests that need a GB300)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libnsgb.so")


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_results.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def cuda_lib():
    """Builds (if stale) and loads the CUDA library; the GPU tests use it."""
    import torch
    from ns_solver_jax_differential_distributed_gb300 import _build, _native
    _build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return _native.lib()


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / (np.linalg.norm(a) + 1e-12))

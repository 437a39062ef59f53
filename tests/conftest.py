import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libkpm kernels)")


def golden(name):
    """Load tests/golden/<name>.npz (fixtures produced by running jclsquant itself)."""
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


@pytest.fixture(scope="session")
def cuda_lib():
    """libkpm loaded on a GPU machine (builds it first if needed)."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test ran without a visible CUDA device")
    from minijclsquant_gb300 import _capi

    return _capi.load(build_if_missing=True)

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    from ogl_beamforming_cuda_gb300 import abi
    return abi.load()


def nrmse_db(x, ref):
    import numpy as np
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.sum(ref ** 2)
    if den == 0:
        return -np.inf if np.sum(x ** 2) == 0 else np.inf
    return 10 * np.log10(max(np.sum((x - ref) ** 2) / den, 1e-300))

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"small_{name}.npz"), allow_pickle=False))


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    from tensormesh_gb300 import _lib
    _lib.load()
    return torch.device("cuda:0")


def rel_fro(a, b):
    import torch
    a = torch.as_tensor(a, dtype=torch.float64).reshape(-1).cpu()
    b = torch.as_tensor(b, dtype=torch.float64).reshape(-1).cpu()
    d = float(torch.linalg.vector_norm(a - b))
    n = float(torch.linalg.vector_norm(b))
    return d / n if n > 0 else d

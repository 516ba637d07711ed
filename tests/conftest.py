import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: longer CPU test")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture
def golden():
    return load_golden


def parse_bc(arr):
    """Fixtures store the BC spec as its repr string."""
    s = str(arr)
    return None if s == "None" else eval(s, {"__builtins__": {}}, {})


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library, for tests marked ``gpu``."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from evoxels_gb300 import _lib
    return _lib.lib()

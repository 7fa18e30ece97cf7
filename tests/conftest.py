import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases(prefix):
    names = sorted(f for f in os.listdir(GOLDEN) if f.startswith(prefix) and f.endswith(".npz"))
    return [n[len(prefix):-4] for n in names]


def load_golden(prefix, name):
    d = np.load(os.path.join(GOLDEN, prefix + name + ".npz"))
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def native_lib():
    from segtaco_gb300 import native
    return native.lib()


@pytest.fixture(scope="session")
def cuda():
    """The GPU path: the CUDA device and the native library, or a hard failure."""
    import torch
    from segtaco_gb300 import native
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    lib = native.lib()
    assert lib.segtaco_device_available() == 1
    return torch.device("cuda:0")

"""Shared fixtures.  `gpu`-marked tests need a CUDA device and call the
product through the C ABI of libfdmgpu.so; the rest run on CPU."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libfdmgpu kernels)")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(GOLDEN / (name + ".npz")))
    return load


@pytest.fixture(scope="session")
def port():
    from fdm_gb300.build import build_oracle
    build_oracle(with_reference=False)
    from oracle.oracle import port as _port
    return _port()


@pytest.fixture(scope="session")
def native():
    """libfdmgpu.so, built here if missing or stale."""
    from fdm_gb300.build import build_cuda
    build_cuda()
    from fdm_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def cuda(native):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")


import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libphono_gpu.so; GPU tests fail loudly without it."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("CUDA device not available for a gpu-marked test")
    from phonomena_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import cpu_oracle

    cpu_oracle.build()
    return cpu_oracle

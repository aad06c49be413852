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


DIV_CHECK_SRC = ROOT / "tests" / "div_gpu.cu"
DIV_CHECK_LIB = ROOT / "tests" / "_build" / "libdivcheck.so"


def build_divcheck():
    """Compile the division-check library (tests/div_gpu.cu: the FP64 path's
    divisor-table code on the host and on the GPU) with the product's nvcc
    flags; test infrastructure, not part of the product build."""
    import subprocess

    from phonomena_gb300 import build

    deps = [DIV_CHECK_SRC, build.CSRC / "div_table.cuh"]
    if not DIV_CHECK_LIB.exists() or any(d.stat().st_mtime > DIV_CHECK_LIB.stat().st_mtime for d in deps):
        DIV_CHECK_LIB.parent.mkdir(exist_ok=True)
        tmp = str(DIV_CHECK_LIB) + ".tmp"
        cmd = [build.nvcc(), *build.ARCH, *build.FLAGS, "-I", str(build.CSRC), "-shared", str(DIV_CHECK_SRC),
               "-o", tmp]
        subprocess.run(cmd, check=True, capture_output=True)
        os.replace(tmp, DIV_CHECK_LIB)
    return DIV_CHECK_LIB

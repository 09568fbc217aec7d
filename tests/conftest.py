import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "square-wheel_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libswgpu.so")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_libs():
    """Build libswgpu.so and the oracle if they are missing (nvcc cross-compiles without a GPU)."""
    import importlib.util
    import subprocess
    spec = importlib.util.spec_from_file_location("swgpu_build", os.path.join(ROOT, "square-wheel_gb300", "build.py"))
    swbuild = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(swbuild)
    swbuild.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j4"], check=True)
    return True


@pytest.fixture(scope="session")
def gpu_ok(built_libs):
    if not _has_gpu():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return True

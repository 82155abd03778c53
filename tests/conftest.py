import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "webgpu-fluid-simulation_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI on the device)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (always) and the CUDA library (cross-compiles without a GPU)."""
    import importlib.util
    for path in (os.path.join(REPO, "oracle", "build.py"), os.path.join(PKG, "build_lib.py")):
        spec = importlib.util.spec_from_file_location("_b_" + os.path.basename(os.path.dirname(path)), path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    yield


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"),
          os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product kernels")


@pytest.fixture(scope="session")
def voce_lib():
    """The product library; built here when missing, never replaced by a
    fallback."""
    from voce_gb300 import build, capi
    if not os.path.exists(capi.LIB_PATH):
        build.build()
    return capi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    if not os.path.exists(oracle.PORT_LIB):
        oracle.build_port()
    return oracle.lib()


def gpu_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return os.path.exists("/dev/nvidia0")

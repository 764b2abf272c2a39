import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    # The native product library and the oracle are built in-tree on first
    # use (both builds are incremental and take seconds).
    from yar_gb300 import build
    build.build_product()
    build.build_oracle()


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx():
    if not cuda_available():
        pytest.skip("no CUDA device")
    from yar_gb300 import native
    ctx = native.Context(0)
    yield ctx
    ctx.close()


def golden(name):
    return os.path.join(GOLDEN, name)

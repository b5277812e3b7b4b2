import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        import subprocess
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library on a visible GPU; GPU tests fail (not skip)
    when the library is missing on a GPU host."""
    if not _gpu_available():
        pytest.skip("no CUDA device")
    import core_gb300
    from core_gb300 import build
    build.build()
    return core_gb300.load()

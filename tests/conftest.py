import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "finch.jl_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds libfinchgb.so if needed and returns the loaded library."""
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from finchgb import _lib, build

    build.build()

    return _lib.load()

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI on the device)")


@pytest.fixture(scope="session")
def core_lib():
    from formura_gb300 import _lib, build

    build.build_library()
    return _lib.lib()


@pytest.fixture(scope="session")
def cuda_device(core_lib):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    assert core_lib.fm_device_count() >= 1
    return torch.device("cuda:0")

"""Test configuration: import paths, the `gpu` marker, and builds of the library and oracle."""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "ff-srl_gb300", ROOT / "oracle", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def built_lib():
    from ffsrl import _build
    return _build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


def _cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(built_lib):
    if not _cuda_ok():
        pytest.fail("test marked gpu but no CUDA device is visible")
    import torch
    return torch.device("cuda:0")

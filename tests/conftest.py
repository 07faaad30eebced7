import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    """libpo_gb300 (built in-tree if missing; no fallback)."""
    from pypo_gb300 import build
    build.build()
    from pypo_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    if not O.LIB_PATH.exists():
        O.build()
    return O


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libraypath.so")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """The in-tree libraypath.so (built on demand, never a fallback)."""
    from europaraypaths_gb300 import build
    build.build()
    from europaraypaths_gb300 import _abi
    return _abi.lib()


@pytest.fixture(scope="session")
def oracle():
    from oracle import loader
    loader.lib()
    return loader


@pytest.fixture
def no_split_parts(built_lib):
    """Split facet parts off for the test (rp_split_parts): a lone small call
    then sums its parts in the same grouping as any larger call, so results
    compare bitwise across call shapes."""
    built_lib.rp_split_parts(0)
    yield
    built_lib.rp_split_parts(1)

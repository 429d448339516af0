import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "oracle"))
sys.path.insert(0, str(REPO / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


@pytest.fixture(scope="session")
def bclbm():
    """The package, with libbclbm.so built (the lattice builder is native too)."""
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return ge.load()


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def native_lib(bclbm):
    """libbclbm.so, built once per session if missing or stale."""
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return bclbm.native.lib()


@pytest.fixture(scope="session")
def gpu(native_lib):
    if not _has_gpu():
        pytest.fail("a test marked gpu ran without a visible CUDA device")
    return native_lib

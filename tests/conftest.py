import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def mhd():
    import heterogeneous_mhd_gb300 as m
    m.lib(build_if_missing=True)
    return m


@pytest.fixture(scope="session")
def oracle32():
    from _oracle import Oracle
    return Oracle(32, "port")


@pytest.fixture(scope="session")
def oracle64():
    from _oracle import Oracle
    return Oracle(64, "port")


@pytest.fixture(scope="session")
def cuda():
    """torch with a visible GPU; GPU tests fail loudly without one."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA GPU is required for -m gpu tests")
    return torch

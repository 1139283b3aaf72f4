import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def lbm_lib():
    """liblbm_gb300.so, built in-tree on first use."""
    from lbm_gb300 import _build, capi
    _build.build()
    return capi.load_library()


@pytest.fixture(scope="session")
def oracle_built():
    import oracle
    oracle.build()
    return oracle

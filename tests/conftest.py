import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


@pytest.fixture(scope="session")
def pkg():
    import ethersph_gb300
    return ethersph_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


@pytest.fixture(scope="session")
def lib():
    """The native library, built in-tree if it is missing or stale."""
    import spfft_gb300
    from spfft_gb300 import build

    build.build()
    return spfft_gb300.load_library()

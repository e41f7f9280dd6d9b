import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def native():
    """The built engine library (built on first use; never a Python fallback)."""
    from subway_gb300 import build, native as nat
    build.build_lib()
    nat.lib()
    return nat


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def gpu(native):
    if native.device_count() < 1:
        pytest.fail("no CUDA device visible: GPU tests need a GB300")
    return native

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the built CUDA library")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built if needed.  GPU tests fail loudly without it."""
    from spp_gb300 import abi, build
    build.build()
    return abi.lib()

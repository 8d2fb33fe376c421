import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a) and the compiled libsphstokes.so")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile the library and the oracle once per session (no-ops when up to date)."""
    from sphericalstokes_gb300.build import build_all

    build_all()
    yield

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libbms.so and the oracle once per session (no-op when up to date)."""
    from bms2_gb300 import build

    build.build()
    yield


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


@pytest.fixture(scope="session")
def ctx():
    from bms2_gb300 import Context

    c = Context(int(os.environ.get("BMS_DEVICE", "0")))
    yield c
    c.close()

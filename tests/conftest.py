import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session", autouse=True)
def _built():
    import __graft_entry__ as g
    from surfacegrowthconsole_gb300 import build as b

    b.build()
    yield


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False

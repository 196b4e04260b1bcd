"""Test configuration: the `gpu` marker, in-tree build once per session, shared helpers."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from backprojector_gb300 import build

    build.build_library()
    build.build_oracle()
    build.build_reference()
    build.build_python_module()
    yield


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")

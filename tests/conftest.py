import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native parts once per session (no-op when up to date)."""
    from pythia_gb300 import _build
    _build.build_datagen()
    _build.build_oracle()
    try:
        _build.build_gpu()
    except Exception as e:  # pragma: no cover - reported by the ABI tests
        print("GPU library build failed:", e)
    return True


@pytest.fixture(scope="session")
def ctx():
    from pythia_gb300 import gpu
    c = gpu.Context(0)
    yield c
    c.close()

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the native libraries in-tree once per session (no-op when fresh)."""
    from titan_gb300 import build
    build.build_library()
    build.build_oracle()
    return True


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture
def omp_threads():
    return int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)

"""Shared test set-up: the `gpu` marker, paths, and the native-library fixtures."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    """librts_scatter.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from relativistic_solver_hllc_gb300 import build_library, load_library

    build_library()
    return load_library()


@pytest.fixture()
def ctx(native_lib):
    from relativistic_solver_hllc_gb300 import Context

    c = Context(0)
    yield c
    c.close()

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libfsgpu.so kernels)")


@pytest.fixture(scope="session")
def ctx():
    """The device context for GPU tests.  No skip: on a GPU host a missing
    device or library is a failure."""
    import flecsolve_gb300 as fs
    c = fs.Context(0)
    yield c
    c.close()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu() -> bool:
    try:
        import ctypes
        from cudagsea_gb300 import _native
        n = ctypes.c_int(0)
        return _native.lib().gsea_device_count(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle and the library once per session (no-op when fresh)."""
    import oracle
    from cudagsea_gb300 import build
    oracle.build()
    build.build()


@pytest.fixture(scope="session")
def gpu():
    if not _has_gpu():
        pytest.fail("a GPU test ran without a usable CUDA device")
    return True

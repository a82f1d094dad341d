import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); parity tests through the C ABI")


@pytest.fixture(scope="session")
def native_lib():
    """The product library, built in-tree if missing (fails loudly, no fallback)."""
    from sharpray_gb300 import _abi
    if not _abi.LIB_PATH.exists():
        from sharpray_gb300.build import build_library
        build_library()
    return _abi.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx(native_lib):
    from sharpray_gb300 import Context
    return Context(0)


@pytest.fixture(scope="session")
def host_ctx(native_lib):
    from sharpray_gb300 import Context
    return Context(-1)


def cpu_threads() -> int:
    return max(1, os.cpu_count() or 1)

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) and runs the CUDA path")


@pytest.fixture(scope="session", autouse=True)
def native_libs():
    """Builds the in-tree libraries once per session (no-op when up to date)."""
    from amat_gb300 import build
    return build.build_all()


@pytest.fixture(scope="session")
def gpu():
    """Skips when the machine has no CUDA device at all; any other failure of
    the device path is an error, never a silent CPU fallback."""
    import ctypes
    from amat_gb300 import libafm
    lib = libafm()
    h = ctypes.c_void_p()
    s = lib.afm_create(ctypes.byref(h), 0, -1)
    if s != 0:
        msg = lib.afm_last_error().decode()
        if "no CUDA device" in msg:
            pytest.skip("no CUDA device on this machine")
        raise RuntimeError("GB300 device path unavailable: " + msg)
    lib.afm_destroy(h)
    return True

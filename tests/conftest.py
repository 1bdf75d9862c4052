import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "massively-parallel-gpu-ode-solver_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    """True when the CUDA driver reports at least one device."""
    import ctypes
    try:
        cuda = ctypes.CDLL("libcuda.so.1")
        if cuda.cuInit(0) != 0:
            return False
        n = ctypes.c_int(0)
        return cuda.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


@pytest.fixture(scope="session")
def native_libs():
    """Build (incrementally) the runtime and every system plugin."""
    from mpgos_gb300 import build
    return build.build_all()


@pytest.fixture(scope="session")
def oracle_libs():
    from oracle import build_oracle
    return build_oracle.build_all()


def golden_files():
    return sorted(GOLDEN.glob("*.npz"))

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda_lib():
    from chemsim_gb300 import build
    build()
    from chemsim_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(cuda_lib):
    """Skips nothing: a GPU test on a machine without a GPU must fail loudly."""
    import ctypes
    from chemsim_gb300 import _lib
    h = ctypes.c_void_p()
    rc = cuda_lib.lbm_create(8, 8, 1.0, 0, 0, ctypes.byref(h))
    if rc != 0:
        raise RuntimeError(f"CUDA lattice creation failed: {_lib.last_error()}")
    cuda_lib.lbm_destroy(h)
    return True

import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def reflib():
    """The reference's shaders compiled as C++; skipped where neither the reference checkout
    nor its generated sources are present (the committed golden fixtures cover that case)."""
    from oracle.oracle import RefLib, build_ref

    try:
        lib = build_ref()
    except Exception as e:  # compiler missing etc.
        pytest.skip(f"reference build failed: {e}")
    if lib is None:
        pytest.skip("reference shaders not available here")
    return RefLib(lib)


@pytest.fixture(scope="session")
def wclib():
    """libwatercube.so (built if stale)."""
    from watercube_gb300.build import build

    build()
    from watercube_gb300 import _abi

    return _abi.lib()


@pytest.fixture(scope="session")
def gpu(wclib):
    import ctypes

    from watercube_gb300 import _abi

    # A 1-particle fluid is the cheapest probe that the CUDA path works on this machine.
    p = _abi.Params()
    wclib.wc_params_dam_break(ctypes.byref(p), 1)
    h = ctypes.c_void_p()
    rc = wclib.wc_fluid_create(ctypes.byref(p), ctypes.byref(h))
    if rc != 0:
        pytest.fail(f"CUDA path unavailable on a GPU test run: {wclib.wc_last_error().decode()}")
    wclib.wc_fluid_destroy(h)
    return True

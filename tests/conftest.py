import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def _have_gpu():
    try:
        r = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=30)
        return r.returncode == 0 and "GPU" in r.stdout
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _have_gpu():
        return
    skip = pytest.mark.skip(reason="no GPU on this host")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def engine_lib():
    """The engine library, compiled if this host has nvcc and it is missing."""
    from wedge_gb300 import build as B

    lib = os.path.join(B.OUT_LIB, B.LIB_NAME)
    if not os.path.exists(lib) or not os.path.exists(os.path.join(B.OUT_BIN, "wedge")):
        B.build_all()
    import wedge_gb300 as W

    W.lib()
    return W

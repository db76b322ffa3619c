import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def reference_root():
    """The reference checkout the CPU tests read input files from: $FE_REFERENCE_ROOT, else
    a directory named ``reference`` beside this repository; None when neither exists."""
    for cand in (os.environ.get("FE_REFERENCE_ROOT"), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.isdir(cand):
            return cand
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def gpu_lib():
    """The built library on a machine with a GPU; GPU tests fail (not skip) without it."""
    from finite_elements_gb300 import _lib
    return _lib.load()

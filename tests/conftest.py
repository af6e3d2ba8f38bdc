import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls libflam3gpu kernels")


@pytest.fixture(scope="session")
def gpulib():
    """libflam3gpu, built in-tree.  GPU tests fail (not skip) when it is missing."""
    from flam3_gb300 import _build, render

    if not os.path.exists(render._LIB_PATH):
        _build.build()
    return render.load()

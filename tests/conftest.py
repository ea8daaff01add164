"""pytest setup: the `gpu` marker, the repository root on sys.path, and the
CPU oracle built before the first test that needs it."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def faces_lib():
    """The built C-ABI library (built here if missing)."""
    import faces_gb300
    if not os.path.isfile(faces_gb300.library_path):
        from faces_gb300 import build
        build.build()
    return faces_gb300

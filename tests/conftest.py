import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests of the CUDA path)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """The oracle library (and the CUDA library, where nvcc is present) must exist before tests run."""
    import __graft_entry__ as g

    if not os.path.exists(os.path.join(ROOT, "oracle", "_build", "libotg_oracle.so")):
        g.build_oracle()
    yield

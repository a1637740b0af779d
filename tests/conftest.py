import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs through the C-ABI library")


@pytest.fixture(scope="session", autouse=True)
def _built_oracle():
    """Build the oracle library (test infrastructure) once per session if missing."""
    from oracle import oracle as _o

    if not os.path.exists(_o.LIB_PATH):
        import subprocess

        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True,
                       capture_output=True)
    yield

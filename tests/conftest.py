import os
import subprocess
import sys

import pytest

# The reference's OpenMP matcher and merge are racy; its single-threaded run is
# the semantics the oracle and the CUDA path reproduce.  Must be set before any
# OpenMP runtime initialises.
os.environ["OMP_NUM_THREADS"] = "1"

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle and the package libraries once per session."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    from cuimg_gb300 import build
    build.build()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger CPU cases")


def pytest_sessionstart(session):
    # the package's compute calls need its compiled library; on a fresh
    # checkout build it first (nvcc cross-compiles for sm_103a without a GPU)
    if os.path.exists(os.path.join(ROOT, "nosh_gb300", "libnosh_gb300.so")):
        return
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "nosh_gb300_build", os.path.join(ROOT, "nosh_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Reference source tree (read only; present in the build container, absent on GPU
# hosts).  Tests that need it skip when it is missing.
os.environ.setdefault("MIEPY_REFERENCE_SRC", "/root/reference/src")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


def reference_available():
    return os.path.isdir(os.path.join(os.environ.get("MIEPY_REFERENCE_SRC", ""), "miepy"))

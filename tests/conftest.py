import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The reference's Python layer, staged into the git-ignored baseline/_ref by
# oracle/stage_reference.py (MIEPY_REFERENCE_SRC overrides it).  Tests that need it
# skip when it is missing.
_STAGED = os.path.join(ROOT, "baseline", "_ref", "src")
if os.path.isdir(os.path.join(_STAGED, "miepy")):
    os.environ.setdefault("MIEPY_REFERENCE_SRC", _STAGED)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


def reference_available():
    return os.path.isdir(os.path.join(os.environ.get("MIEPY_REFERENCE_SRC", ""), "miepy"))

"""Stage the reference's Python package and test files into ``baseline/_ref``.

TEST INFRASTRUCTURE ONLY.  The reference (johnaparker/miepy) cannot be installed
as a package here: its native module needs Eigen, GSL and a vcpkg checkout that
are absent, so ``pip install --target baseline/_ref`` stops at the CMake step.
Its Python layer (``src/miepy``) and test files (``tests/``) run unmodified on the
oracle (``oracle/refshim.py`` registers the oracle as ``miepy.cpp``), so this
recipe copies those two trees, byte for byte, into the git-ignored
``baseline/_ref`` (``baseline/_ref/src/miepy``, ``baseline/_ref/tests``).  The
staged tree is never committed; it travels with the working copy to GPU hosts,
where the reference tree itself is absent, so that the tests that run the
reference's own ``sphere_cluster`` through this package's plugin can run there.

Usage:  python oracle/stage_reference.py [reference checkout]
        (default: /root/reference; does nothing if that checkout is absent)
"""

from __future__ import annotations

import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEST = os.path.join(ROOT, "baseline", "_ref")
DEFAULT_SRC = "/root/reference"

_SKIP = shutil.ignore_patterns("__pycache__", "*.pyc", "*.so", "*.pyd", ".pytest_cache")


def _newest(tree: str) -> float:
    t = 0.0
    for d, _, files in os.walk(tree):
        for f in files:
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def stage(ref: str = DEFAULT_SRC) -> str | None:
    """Copy ``<ref>/src/miepy`` and ``<ref>/tests`` under ``baseline/_ref``.

    Returns the staged ``src`` directory, or None when the reference checkout is
    absent (GPU hosts: an earlier staging travelled with the working copy)."""
    pkg = os.path.join(ref, "src", "miepy")
    tests = os.path.join(ref, "tests")
    if not (os.path.isdir(pkg) and os.path.isdir(tests)):
        return None
    for src, dst in ((pkg, os.path.join(DEST, "src", "miepy")), (tests, os.path.join(DEST, "tests"))):
        if os.path.isdir(dst) and _newest(dst) >= _newest(src):
            continue
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        shutil.copytree(src, dst, ignore=_SKIP)
    return os.path.join(DEST, "src")


if __name__ == "__main__":
    out = stage(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_SRC)
    print(out if out else "reference checkout not found; nothing staged")

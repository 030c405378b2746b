"""Pin the oracle with the reference's own test suite.

The reference's test files (physics identities, the FDTD golden data, Gaussian
beam power, far/near-field identities ...) are executed unmodified by pytest, with
the oracle registered as ``miepy.cpp``.  Needs the reference source tree, so it
skips where that tree is absent (GPU hosts)."""

import os
import subprocess
import sys

import pytest

from tests.conftest import ROOT, reference_available

# Reference test files on the sphere-cluster path that the oracle must pass, with
# the expected number of passing tests.
PINNED = {
    "test_single_gmt.py": 3,
    "test_cluster.py": 2,
    "test_vsh_translation.py": 0,      # asserts at import time
    "test_cluster_coefficients.py": 2,
    "test_cross_sections.py": 2,
    "test_force.py": 2,
    "test_fdtd_comparison.py": 2,
    "test_far_field.py": 3,
    "test_fields.py": 1,
    "test_medium.py": 2,
    "test_near_to_far.py": 7,
    "test_decomposition.py": 1,
    "test_beam_power.py": 11,
    "test_weak_focusing.py": 6,
    "test_tight_focusing.py": 8,
    "test_poynting_vector.py": 6,
    "test_point_matching.py": 2,
    "test_coordinate_geometry.py": 2,
    "test_source_rotation.py": 1,
    "test_interface.py": 4,
    "test_maxwells_equations.py": 14,
}

# Parametrisations deselected by a -k expression on their ids (none at present: the
# Gaussian-beam cases of test_interface.py, which rotate expansion coefficients, run
# with the harness's stand-in for the ``spherical`` package).
DESELECT = {}

pytestmark = pytest.mark.skipif(not reference_available(), reason="reference source tree not available")


@pytest.mark.parametrize("fname", sorted(PINNED))
def test_reference_suite_passes_on_oracle(fname):
    ref_tests = os.path.join(os.path.dirname(os.environ["MIEPY_REFERENCE_SRC"]), "tests", fname)
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    cmd = [sys.executable, "-m", "pytest", "-p", "no:cacheprovider", "-p", "oracle.pytest_refshim", "-q",
           "--rootdir", ROOT, ref_tests]
    if fname in DESELECT:
        cmd += ["-k", DESELECT[fname]]
    res = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    tail = res.stdout[-2000:] + res.stderr[-2000:]
    expected = PINNED[fname]
    if expected == 0:
        assert res.returncode in (0, 5), tail   # 5 = no tests collected (import-time asserts passed)
    else:
        assert res.returncode == 0, tail
        assert f"{expected} passed" in res.stdout, tail

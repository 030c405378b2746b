"""Loader for the golden fixtures in tests/golden (made by tests/golden/make_golden.py)."""

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CASES = ["dimer_lmax6_exact", "dimer_lmax6_bicgstab", "ag5_lmax2_exact", "ag5_lmax2_bicgstab",
         "rand12_lmax3_exact", "rand4_lmax8_exact", "drude2_lmax4_450nm_exact", "drude2_lmax4_800nm_exact",
         "gauss3_lmax3_exact"]
EXACT_CASES = [c for c in CASES if c.endswith("_exact")]


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}

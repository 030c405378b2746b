"""Gaussian-beam source decomposition against the reference's own result.

Fixture gauss_beam_lmax5 holds gaussian_beam(width=1 um, polarization=[1, 0]).structure
at 7 points, lmax 5, 600 nm in vacuum, computed by the reference's Python
(sources/beams.py:168-200 -> vsh/decomposition.py:284-325 -> integrate_phase).
CPU: the host far-field projection, summed in numpy, reproduces it (rtol 1e-12 of the
largest coefficient).  GPU: gb_beam_project reproduces it (same bar), and a cluster
driven by the beam matches the exact fixture gauss3_lmax3_exact.
"""

import numpy as np
import pytest

from miepy_gb300.beams import gaussian_beam
from tests import _golden as G

nm = 1e-9


def _beam(g):
    return gaussian_beam(width=float(g["width"]), polarization=g["polarization"])


def test_beam_constants_match_reference():
    g = G.load("gauss_beam_lmax5")
    b = _beam(g)
    k = float(g["k"])
    assert abs(b.E0(k) - float(g["E0"])) <= 1e-13 * abs(float(g["E0"]))
    assert abs(b.theta_cutoff(k) - float(g["theta_c"])) <= 1e-15


def test_far_projection_reproduces_reference_structure():
    g = G.load("gauss_beam_lmax5")
    b = _beam(g)
    k, L = float(g["k"]), int(g["lmax"])
    rhat, w = b.far_projection(k, L)
    pos = g["position"]
    ph = np.exp(-1j * k * (pos @ rhat.T))               # [N, G]
    p = (ph @ w).reshape(pos.shape[0], 2, -1)
    ref = g["p_src"]
    assert np.max(np.abs(p - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_device_beam_projection_matches_reference():
    g = G.load("gauss_beam_lmax5")
    b = _beam(g)
    p = b.structure(g["position"], float(g["k"]), int(g["lmax"]))
    ref = g["p_src"]
    assert np.max(np.abs(p - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_cluster_driven_by_gaussian_beam():
    import miepy_gb300 as gb
    g = G.load("gauss3_lmax3_exact")
    src = gaussian_beam(width=1000 * nm, polarization=[1, 0])
    c = gb.sphere_cluster(position=g["position"], radius=g["radius"],
                          material=gb.constant_material(index=1.5 + 0.01j), source=src,
                          wavelength=float(g["wavelength"]), lmax=int(g["lmax"]), method=gb.solver.exact)
    assert np.max(np.abs(c.p_src - g["p_src"])) <= 1e-12 * np.max(np.abs(g["p_src"]))
    np.testing.assert_allclose(c.p_inc, g["p_inc"], rtol=1e-10, atol=1e-14 * np.max(np.abs(g["p_inc"])))
    C = c.cross_sections()
    ref = g["cross_sections"]
    assert abs(C.extinction - ref[2]) <= 1e-9 * abs(ref[2])
    np.testing.assert_allclose(c.force(), g["force"], rtol=1e-9, atol=1e-9 * np.max(np.abs(g["force"])))

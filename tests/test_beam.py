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


# ----------------------------------------------------- rotated and reflected --
def test_rotation_of_a_plane_wave_matches_its_direct_decomposition():
    """The Wigner-D rotation (miepy_gb300.rotation) of the +z plane wave's
    coefficients, taken at the positions in the rotated frame, equals the direct
    decomposition of the plane wave at (theta, phi): 1e-13 of the largest
    coefficient, lmax 7, three polarisations, four directions (CPU)."""
    import miepy_gb300 as gb
    from miepy_gb300 import rotation as ROT
    k = 2 * np.pi / (600 * nm)
    pos = np.random.default_rng(0).uniform(-300 * nm, 300 * nm, size=(5, 3))
    for pol in ([1, 0], [0, 1], [1, 1j]):
        for th, ph in ((0.3, 0.0), (0.7, 1.1), (2.5, -0.4), (np.pi, 0.2)):
            direct = gb.plane_wave(polarization=pol, theta=th, phi=ph).structure(pos, k, 7)
            frame = pos @ ROT.rotation_matrix(ph, th)
            p = ROT.rotate_expansion_coefficients(gb.plane_wave(polarization=pol).structure(frame, k, 7), ph, th)
            assert np.max(np.abs(p - direct)) <= 1e-13 * np.max(np.abs(direct))


@pytest.mark.gpu
def test_rotated_beams_match_reference():
    """Fixture gauss_beam_rotated_lmax5: the reference's rotated beams (its beam
    decomposition and coefficient rotation, with the harness's Wigner-D), 1e-11."""
    g = G.load("gauss_beam_rotated_lmax5")
    k, L = float(g["k"]), int(g["lmax"])
    for q in range(3):
        b = gaussian_beam(width=float(g["width"]), polarization=g[f"polarization_{q}"], theta=float(g[f"theta_{q}"]),
                          phi=float(g[f"phi_{q}"]), center=g[f"center_{q}"])
        p = b.structure(g["position"], k, L)
        ref = g[f"p_src_{q}"]
        assert np.max(np.abs(p - ref)) <= 1e-11 * np.max(np.abs(ref)), q


@pytest.mark.gpu
def test_beam_polarisation_turns_with_phi():
    """A beam along +z rotated by phi about z is the beam whose polarisation is
    turned by phi (an identity between the rotation and the angular spectrum)."""
    k = 2 * np.pi / (600 * nm)
    pos = np.random.default_rng(3).uniform(-500 * nm, 500 * nm, size=(6, 3))
    for phi in (0.4, 2.1):
        a = gaussian_beam(width=1000 * nm, polarization=[1, 0], phi=phi).structure(pos, k, 5)
        b = gaussian_beam(width=1000 * nm, polarization=[np.cos(phi), np.sin(phi)]).structure(pos, k, 5)
        assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(b))


@pytest.mark.gpu
def test_beam_above_interface_matches_reference():
    """Fixture interface_gauss3_lmax3_exact: the substrate trimer driven by a
    Gaussian beam, whose source includes the reflected beam: p_src and p_inc 1e-10,
    cross-sections, forces and torques 1e-9."""
    import miepy_gb300 as gb
    g = G.load("interface_gauss3_lmax3_exact")
    sub = gb.interface(gb.constant_material(index=1.7), z=-120 * nm)
    c = gb.sphere_cluster(position=g["position"], radius=g["radius"], material=gb.constant_material(index=1.5 + 0.01j),
                          medium=gb.materials.water(), source=gaussian_beam(width=1000 * nm, polarization=[1, 0]),
                          wavelength=600 * nm, lmax=3, interface=sub, method=gb.solver.exact)
    assert np.max(np.abs(c.p_src - g["p_src"])) <= 1e-10 * np.max(np.abs(g["p_src"]))
    np.testing.assert_allclose(c.p_inc, g["p_inc"], rtol=1e-10, atol=1e-14 * np.max(np.abs(g["p_inc"])))
    C = c.cross_sections()
    np.testing.assert_allclose([C.scattering, C.absorption, C.extinction], g["cross_sections"], rtol=1e-9)
    F, T = c.force(), c.torque()
    assert np.max(np.abs(F - g["force"])) <= 1e-9 * np.max(np.abs(g["force"]))
    assert np.max(np.abs(T - g["torque"])) <= 1e-9 * np.max(np.abs(g["torque"]))

"""Planar interface (substrate): reflected source, reflection matrix, solve.

Pinned by the fixture ``interface3_lmax3_exact`` (a trimer 120 nm above an n = 1.7
half-space in water, plane wave, lmax 3), made by the reference's own Python
(tests/golden/make_golden.py), and by the reference's interface identities
(tests/test_interface.py of the reference: translating the interface together
with the particles, an index-matched interface).

CPU: the oracle's reflection matrix and the host-side reflected plane wave against
the fixture.  GPU: gb_reflection_matrix_dense against the fixture (1e-12 of the
largest entry), the cluster solve (p_inc 1e-10, cross-sections / forces / torques /
fields 1e-9) and the two identities.
"""

import numpy as np
import pytest

from tests import _golden as G

nm = 1e-9


def fixture():
    return G.load("interface3_lmax3_exact")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(np.asarray(b))))


def test_oracle_reflection_matrix_matches_fixture():
    from oracle import oracle as O
    g = fixture()
    R = O.reflection_matrix_nia(g["position"], g["mie_scat"], g["k_b"], g["r0"], g["interface_z"])
    assert rel(R, g["reflection_matrix"].reshape(R.shape)) < 1e-13


def test_reflected_plane_wave_source():
    import miepy_gb300 as gb
    g = fixture()
    medium = gb.materials.water() if hasattr(gb.materials, "water") else gb.constant_material(index=1.33)
    sub = gb.interface(gb.constant_material(index=complex(g["interface_index"])), z=float(g["interface_z"]))
    src = gb.plane_wave([1, 0])
    r0 = sub.reflection_coefficients(0, float(g["wavelength"]), medium)[0]
    assert abs(r0 - g["r0"]) < 1e-14
    k = float(g["k_b"])
    lmax = int(g["lmax"])
    p = src.structure(g["position"], k, lmax) + src.reflect(sub, medium, float(g["wavelength"])).structure(
        g["position"], k, lmax)
    assert rel(p, g["p_src"]) < 1e-12


@pytest.mark.gpu
def test_reflection_matrix_on_gpu():
    from miepy_gb300 import backend
    g = fixture()
    R = backend.reflection_matrix_nia(g["position"], g["mie_scat"], g["k_b"], g["r0"], g["interface_z"])
    assert rel(R, g["reflection_matrix"]) < 1e-12


def _cluster(g, **kw):
    import miepy_gb300 as gb
    medium = gb.materials.water() if hasattr(gb.materials, "water") else gb.constant_material(index=1.33)
    sub = gb.interface(gb.constant_material(index=complex(g["interface_index"])), z=float(g["interface_z"]))
    return gb.sphere_cluster(position=g["position"], radius=g["radius"],
                             material=gb.constant_material(index=1.5 + 0.01j), medium=medium,
                             source=gb.plane_wave([1, 0]), wavelength=float(g["wavelength"]), lmax=int(g["lmax"]),
                             interface=sub, **kw)


@pytest.mark.gpu
def test_cluster_with_interface_matches_fixture():
    import miepy_gb300 as gb
    g = fixture()
    c = _cluster(g, method=gb.solver.exact)
    assert rel(c.p_src, g["p_src"]) < 1e-12
    assert rel(c.p_inc, g["p_inc"]) < 1e-10
    C = c.cross_sections()
    np.testing.assert_allclose([C.scattering, C.absorption, C.extinction], g["cross_sections"], rtol=1e-9)
    assert rel(c.force(), g["force"]) < 1e-9
    assert rel(c.torque(), g["torque"]) < 1e-9
    E = c.E_field(g["field_x"], g["field_y"], g["field_z"])
    assert rel(E, g["E_total"]) < 1e-9
    # BiCGSTAB on the dense operator reaches the same p_inc
    cb = _cluster(g, tol=1e-12)
    assert cb.solver_status == 0
    assert rel(cb.p_inc, g["p_inc"]) < 1e-9


@pytest.mark.gpu
def test_interface_identities():
    """The reference's identities (tests/test_interface.py): moving particle and source
    together with the interface leaves the cross-sections unchanged (to 7e-4 for this
    metallic sphere, in the reference as here: both triples are pinned to the
    reference's values, fixture interface_identity); an index-matched interface is no
    interface."""
    import miepy_gb300 as gb
    ref = G.load("interface_identity")
    medium = gb.constant_material(index=1.33)
    mat = gb.constant_material(index=0.2 + 3.0j)
    kw = dict(radius=75 * nm, material=mat, medium=medium, lmax=2, wavelength=600 * nm, method=gb.solver.exact)
    z = 400 * nm
    c1 = gb.sphere_cluster(position=[0, 0, -z], source=gb.plane_wave([1, 0]),
                           interface=gb.interface(gb.constant_material(index=1.7)), **kw)
    c2 = gb.sphere_cluster(position=[0, 0, 0], source=gb.plane_wave([1, 0]),
                           interface=gb.interface(gb.constant_material(index=1.7), z=z), **kw)
    np.testing.assert_allclose(np.array(c1.cross_sections()), ref["C1"], rtol=1e-9)
    np.testing.assert_allclose(np.array(c2.cross_sections()), ref["C2"], rtol=1e-9)
    np.testing.assert_allclose(np.array(c1.cross_sections()), np.array(c2.cross_sections()), rtol=1e-3, atol=0)
    kw.pop("method")
    c3 = gb.sphere_cluster(position=[[0, 0, 0], [200 * nm, 0, 50 * nm]], source=gb.plane_wave([1, 0]),
                           interface=gb.interface(medium, z=-z), tol=1e-12, **kw)
    c4 = gb.sphere_cluster(position=[[0, 0, 0], [200 * nm, 0, 50 * nm]], source=gb.plane_wave([1, 0]), tol=1e-12, **kw)
    np.testing.assert_allclose(np.array(c3.cross_sections()), np.array(c4.cross_sections()), rtol=1e-9, atol=0)

"""Periodic clusters: the lattice sums of sphere_aggregate_tmatrix_periodic.

Pinned by two fixtures made by the reference's own Python (tests/golden/
make_golden.py): ``interactions.sphere_aggregate_tmatrix_periodic``
(interactions.py:153-186, lattice sums over ``symmetry.generate(5000)``) and
``sphere_cluster(symmetry=..., method=exact)`` (sphere_cluster.py:694-712) for a
dimer in a 700 nm square lattice under an oblique plane wave (lmax 2, 5040 cells)
and for one sphere in a 450 nm chain along x (lmax 3, 5000 cells).

CPU: the lattice generators give the reference's cells; the oracle's periodic
aggregate and its dense solve reproduce the fixtures.  GPU:
gb_aggregate_periodic_dense against the fixture (1e-12 of the largest entry) and
the periodic sphere_cluster (p_inc 1e-10; cross-sections, forces, torques 1e-9),
with the exact and the BiCGSTAB solve.
"""

import numpy as np
import pytest

from tests import _golden as G

nm = 1e-9
CASES = {
    "periodic_square_dimer_lmax2": ("square_lattice_2d", 700 * nm, dict(polarization=[1, 0.5j], theta=0.35, phi=0.6)),
    "periodic_chain_single_lmax3": ("x_translation_1d", 450 * nm, dict(polarization=[0, 1], theta=0.5, phi=0.0)),
}


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(np.asarray(b))))


def lattice(name):
    import miepy_gb300 as gb
    kind, a, _ = CASES[name]
    return getattr(gb.symmetry, kind)(a)


@pytest.mark.parametrize("name", list(CASES))
def test_lattice_cells_are_the_references(name):
    g = G.load(name)
    x, y, z = lattice(name).generate(5000)
    cells = np.array([x, y, z]).T
    assert cells.shape == g["cells"].shape
    a, b = np.lexsort(cells.T), np.lexsort(g["cells"].T)
    assert np.max(np.abs(cells[a] - g["cells"][b])) < 1e-12 * np.max(np.abs(g["cells"]))


def test_y_and_z_chains_are_the_x_chain_rotated():
    import miepy_gb300 as gb
    x = np.array(gb.symmetry.x_translation_1d(3.0).generate(10))
    y = np.array(gb.symmetry.y_translation_1d(3.0).generate(10))
    z = np.array(gb.symmetry.z_translation_1d(3.0).generate(10))
    np.testing.assert_array_equal(y, x[[1, 0, 2]])
    np.testing.assert_array_equal(z, x[[2, 1, 0]])


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_periodic_aggregate_and_solve(name):
    from oracle import oracle as O
    g = G.load(name)
    A = O.sphere_aggregate_tmatrix_periodic(g["position"], g["mie_scat"], g["k_b"], g["cells"], g["k_hat"])
    assert rel(A, g["agg_tmatrix"].reshape(A.shape)) < 1e-13
    D = A.shape[0]
    p = np.linalg.solve(np.eye(D) + A, g["p_src"].reshape(-1))
    assert rel(p, g["p_inc"].reshape(-1)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_periodic_aggregate_on_gpu(name):
    from miepy_gb300 import backend
    g = G.load(name)
    A = backend.sphere_aggregate_tmatrix_periodic(g["position"], g["mie_scat"], g["k_b"], lattice(name), g["k_hat"])
    assert rel(A, g["agg_tmatrix"]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("method", ["exact", "bicgstab"])
def test_periodic_sphere_cluster(name, method):
    import miepy_gb300 as gb
    g = G.load(name)
    _, _, src = CASES[name]
    src = dict(src)
    c = gb.sphere_cluster(position=g["position"], radius=g["radius"], material=gb.constant_material(index=1.8 + 0.02j),
                          medium=gb.constant_material(index=1.33), source=gb.plane_wave(src.pop("polarization"), **src),
                          wavelength=float(g["wavelength"]), lmax=int(g["lmax"]), symmetry=lattice(name),
                          method=getattr(gb.solver, method), tol=None if method == "exact" else 1e-13)
    assert c.solver_status == 0
    assert rel(c.p_src, g["p_src"]) < 1e-12
    assert rel(c.p_inc, g["p_inc"]) < 1e-10
    assert rel(c.p_scat, g["p_scat"]) < 1e-10
    C = c.cross_sections()
    np.testing.assert_allclose([C.scattering, C.absorption, C.extinction], g["cross_sections"], rtol=1e-9)
    assert rel(c.force(), g["force"]) < 1e-9
    assert rel(c.torque(), g["torque"]) < 1e-9


@pytest.mark.gpu
def test_periodic_cluster_above_an_interface():
    """symmetry= and interface= together: the lattice sums minus the reflection
    matrix (sphere_cluster.py:694-710), against the reference's own solve."""
    import miepy_gb300 as gb
    g = G.load("periodic_interface_dimer_lmax2")
    c = gb.sphere_cluster(position=g["position"], radius=g["radius"], material=gb.constant_material(index=2.0 + 0.05j),
                          medium=gb.constant_material(index=1.33), source=gb.plane_wave([1, 0]),
                          wavelength=float(g["wavelength"]), lmax=2, symmetry=gb.symmetry.square_lattice_2d(650 * nm),
                          interface=gb.interface(gb.constant_material(index=1.6), z=-150 * nm), method=gb.solver.exact)
    assert rel(c.p_src, g["p_src"]) < 1e-12
    assert rel(c.p_inc, g["p_inc"]) < 1e-10
    C = c.cross_sections()
    np.testing.assert_allclose([C.scattering, C.absorption, C.extinction], g["cross_sections"], rtol=1e-9)
    assert rel(c.force(), g["force"]) < 1e-9
    assert rel(c.torque(), g["torque"]) < 1e-9

"""The drop-in through the reference's own dispatch.

The reference's Python layer (staged into baseline/_ref by
oracle/stage_reference.py, unmodified, with the oracle standing in for its
compiled miepy.cpp) is switched to this package with ``miepy_gb300.backend.install()``
and ``miepy.backends.set_backend('gpu')``.  The reference's own
``miepy.sphere_cluster`` then calls the three plugin names at its dispatch sites
(interactions.py:81-83,141-143, flux.py:21-26), assigns the solve in place
(``self.p_inc[...] = ...``, sphere_cluster.py:713) and, above a substrate, edits
the returned aggregate (``agg -= R``, sphere_cluster.py:709).

Cases (method=solver.exact, the plugin's BiCGSTAB to 1e-14), against the
reference's own exact solves in the golden fixtures: the water dimer at lmax 6
(config 1), the Ag pentamer at lmax 2, and the trimer above an n = 1.7
half-space.  Bars: p_inc and p_scat rtol 1e-10 (atol 1e-14 of the largest
coefficient), cross-sections (computed by the reference through the plugin's
particle_cross_sections_jax) 1e-9, forces and torques 1e-9 of the largest entry.
The library's launch counter shows its kernels ran.
"""

import numpy as np
import pytest

from miepy_gb300 import _native as nat
from tests import _golden as G
from tests.conftest import reference_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not reference_available(), reason="reference Python layer not staged")]

nm = 1e-9


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(np.asarray(b))), 1e-300))


@pytest.fixture(scope="module")
def miepy_gpu():
    from oracle.refshim import import_reference
    from miepy_gb300 import backend

    miepy = import_reference()
    backend.install()
    miepy.backends.set_backend("gpu")
    try:
        yield miepy
    finally:
        miepy.backends.set_backend("cpu")


def _check(c, g):
    for k in ("p_inc", "p_scat"):
        np.testing.assert_allclose(c.__dict__[k], g[k], rtol=1e-10, atol=1e-14 * np.max(np.abs(g[k])))
    C = c.cross_sections()
    np.testing.assert_allclose([C.scattering, C.absorption, C.extinction], g["cross_sections"], rtol=1e-9)
    assert rel(c.force(), g["force"]) < 1e-9
    assert rel(c.torque(), g["torque"]) < 1e-9


def _runs_on_gpu(build):
    L = nat.lib()
    before = L.gb_launch_count()
    c = build()
    assert L.gb_launch_count() > before   # the plugin's kernels ran
    return c


def test_dimer_lmax6_through_reference_dispatch(miepy_gpu):
    miepy = miepy_gpu
    assert miepy.backends.get_backend() == "gpu"
    g = G.load("dimer_lmax6_exact")
    c = _runs_on_gpu(lambda: miepy.sphere_cluster(
        position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
        material=miepy.constant_material(index=0.2 + 3.0j), source=miepy.sources.plane_wave.from_string(polarization="x"),
        wavelength=600 * nm, lmax=6, medium=miepy.materials.water(), method=miepy.solver.exact))
    _check(c, g)


def test_ag_pentamer_through_reference_dispatch(miepy_gpu):
    miepy = miepy_gpu
    g = G.load("ag5_lmax2_exact")
    five = [[0, 0, 0], [250 * nm, 0, 0], [-250 * nm, 0, 0], [0, 250 * nm, 0], [0, -250 * nm, 0]]
    c = _runs_on_gpu(lambda: miepy.sphere_cluster(
        position=five, radius=75 * nm, material=miepy.materials.Ag(),
        source=miepy.sources.plane_wave.from_string(polarization="rhc"), wavelength=600 * nm, lmax=2,
        method=miepy.solver.exact))
    _check(c, g)


def test_interface_trimer_edits_the_plugin_aggregate(miepy_gpu):
    miepy = miepy_gpu
    g = G.load("interface3_lmax3_exact")
    sub = miepy.interface(miepy.constant_material(index=1.7), z=-120 * nm)
    c = _runs_on_gpu(lambda: miepy.sphere_cluster(
        position=[[0, 0, 0], [210 * nm, 40 * nm, 30 * nm], [-160 * nm, 90 * nm, 60 * nm]],
        radius=[70 * nm, 60 * nm, 80 * nm], material=miepy.constant_material(index=1.5 + 0.01j),
        medium=miepy.materials.water(), source=miepy.sources.plane_wave([1, 0]), wavelength=600 * nm, lmax=3,
        interface=sub, method=miepy.solver.exact))
    _check(c, g)

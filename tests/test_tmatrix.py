"""General particles given by T-matrices (the reference's miepy.cluster).

Pinned by the fixture ``tmatrix3_lmax3_exact``: the reference's own ``miepy.cluster``
(cluster.py:16-112, 629-657) with a sphere, a core-shell particle and a particle
whose T-matrix has dense random blocks, lmax 3, in water, a circularly polarised
plane wave, exact solve (tests/golden/make_golden.py).  The oracle's
``particle_aggregate_tmatrix`` (interactions.cpp:417-462) is pinned against its
sphere restatement, which the reference's own tests pin.

CPU: the oracle's aggregate with sphere T-matrices equals the sphere aggregate; the
oracle's dense solve reproduces the reference cluster; the host T-matrix of a
sphere equals the reference's.  GPU: the dense aggregate (1e-12 of the largest
entry), the cluster solve against the fixture (p_inc 1e-10; cross-sections,
forces, torques 1e-9), the mixed-precision solve (C_ext 1e-6), sphere T-matrices
against sphere_cluster, and batch reuse through load().
"""

import numpy as np
import pytest

from tests import _golden as G

nm = 1e-9


def fixture():
    return G.load("tmatrix3_lmax3_exact")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(np.asarray(b))))


def sphere_tmatrices(mie_scat):
    """[N, 2, lmax] Mie coefficients -> diagonal T-matrices [N, 2, rmax, 2, rmax]."""
    N, _, L = mie_scat.shape
    rmax = L * (L + 2)
    n_of_r = np.concatenate([[n] * (2 * n + 1) for n in range(1, L + 1)])
    T = np.zeros((N, 2, rmax, 2, rmax), dtype=complex)
    idx = np.arange(rmax)
    T[:, 0, idx, 0, idx] = mie_scat[:, 0, n_of_r - 1]
    T[:, 1, idx, 1, idx] = mie_scat[:, 1, n_of_r - 1]
    return T


def random_cluster(seed, N=6, lmax=3):
    import miepy_gb300 as gb
    rng = np.random.default_rng(seed)
    pos = np.array([[0, 0, 0]] + [[0, 0, 0]] * (N - 1), dtype=float)
    for i in range(1, N):
        while True:
            p = rng.uniform(-350, 350, 3) * nm
            if np.min(np.linalg.norm(pos[:i] - p, axis=1)) > 190 * nm:
                pos[i] = p
                break
    radius = rng.uniform(60, 85, N) * nm
    eps = (rng.uniform(1.5, 2.5, N) + 0.05j) ** 2
    k = 2 * np.pi * 1.33 / (620 * nm)
    mie, _ = gb.mie_coefficients(radius, eps, 1.0, 1.33 ** 2, 1.0, k, lmax)
    return pos, radius, eps, mie, k


class fixed_particle:
    """A particle with a given T-matrix (what the reference's particle classes provide)."""

    def __init__(self, position, tmatrix, enclosed=None):
        self.position = np.asarray(position, dtype=float)
        self._T = tmatrix
        self._r = enclosed

    def compute_tmatrix(self, lmax, wavelength, eps_m, **kw):
        return self._T

    def enclosed_radius(self):
        return self._r


# ------------------------------------------------------------------------ CPU --
def test_oracle_particle_aggregate_with_sphere_tmatrices_is_the_sphere_aggregate():
    from oracle import oracle as O
    pos, _, _, mie, k = random_cluster(3)
    A_sph = O.sphere_aggregate_tmatrix(pos, mie, k)
    A_gen = O.particle_aggregate_tmatrix(pos, sphere_tmatrices(mie), k)
    assert rel(A_gen, A_sph) < 1e-13


def test_oracle_solve_reproduces_reference_cluster():
    from oracle import oracle as O
    g = fixture()
    A = O.particle_aggregate_tmatrix(g["position"], g["tmatrix"], g["k_b"])
    assert rel(A, g["agg_tmatrix"].reshape(A.shape)) < 1e-13
    D = g["p_src"].size
    p = np.linalg.solve(np.eye(D) + A.reshape(D, D), g["p_src"].reshape(-1)).reshape(g["p_src"].shape)
    assert rel(p, g["p_inc"]) < 1e-10
    assert rel(np.einsum("naibj,nbj->nai", g["tmatrix"], p), g["p_scat"]) < 1e-10


def test_sphere_tmatrix_and_source_match_reference():
    import miepy_gb300 as gb
    g = fixture()
    T = gb.tmatrix_sphere(70 * nm, 600 * nm, (1.9 + 0.05j) ** 2, 1.33 ** 2, 3)
    assert rel(T, g["tmatrix"][0]) < 1e-12
    p = gb.plane_wave([1, 1j]).structure(g["position"], float(g["k_b"]), 3)
    assert rel(p, g["p_src"]) < 1e-12


# ------------------------------------------------------------------------ GPU --
@pytest.mark.gpu
def test_dense_particle_aggregate_on_gpu():
    from miepy_gb300 import backend
    g = fixture()
    A = backend.particle_aggregate_tmatrix(g["position"], g["tmatrix"], g["k_b"])
    assert rel(A, g["agg_tmatrix"]) < 1e-12
    pos, _, _, mie, k = random_cluster(5, N=9, lmax=4)
    rng = np.random.default_rng(1)
    T = sphere_tmatrices(mie) + 0.02 * (rng.standard_normal((9, 2, 24, 2, 24)) + 1j * rng.standard_normal((9, 2, 24, 2, 24)))
    from oracle import oracle as O
    A = backend.particle_aggregate_tmatrix(pos, T, k)
    assert rel(A.reshape(432, 432), O.particle_aggregate_tmatrix(pos, T, k).reshape(432, 432)) < 1e-12


@pytest.mark.gpu
def test_tmatrix_cluster_lmax9_on_the_dense_operator():
    """A cluster of general particles at lmax 9 (beyond the packed solvers' lmax 8)
    solves on the dense aggregate: p_inc within 1e-10 of numpy's direct solve of the
    oracle's aggregate, p_scat = T p_inc, and C_ext against the oracle's
    cross-sections (1e-9).  The T-matrices are the spheres' with a cross-polarised
    coupling of the dipole and quadrupole orders, so that they are not diagonal."""
    import miepy_gb300 as gb
    from oracle import oracle as O
    N, lmax = 3, 9
    rmax = lmax * (lmax + 2)
    pos, radius, eps, mie, k = random_cluster(9, N=N, lmax=lmax)
    rng = np.random.default_rng(4)
    T = sphere_tmatrices(mie)
    c8 = 0.01 * (rng.standard_normal((N, 8, 8)) + 1j * rng.standard_normal((N, 8, 8)))
    T[:, 0, :8, 1, :8] += c8
    T[:, 1, :8, 0, :8] += c8.transpose(0, 2, 1)
    parts = [fixed_particle(pos[i], T[i], radius[i]) for i in range(N)]
    with pytest.warns(UserWarning, match="lmax > 8"):
        c = gb.cluster(particles=parts, source=gb.plane_wave([1, 1j]), wavelength=620 * nm, lmax=lmax,
                       medium=gb.constant_material(index=1.33), method=gb.solver.exact, precision="mixed")
    assert c.solver_status == 0
    b = c._batch   # the dense route allocates no packed matrix
    assert not b.packed and b.mat128 is None and b.mat64 is None
    with pytest.raises(ValueError, match="packed=False"):
        b.assemble()
    D = 2 * rmax * N
    A = O.particle_aggregate_tmatrix(pos, T, k).reshape(D, D)
    x = np.linalg.solve(np.eye(D) + A, c.p_src.reshape(-1)).reshape(N, 2, rmax)
    assert rel(c.p_inc, x) < 1e-10
    assert rel(c.p_scat, np.einsum("naibj,nbj->nai", T, x)) < 1e-10
    per = [O.particle_cross_sections(c.p_scat[i], c.p_inc[i], c.p_src[i], k) for i in range(N)]
    cext = sum(np.sum(p[2]) for p in per)
    assert abs(c.cross_sections().extinction - cext) <= 1e-9 * abs(cext)


def _reference_cluster(**kw):
    import miepy_gb300 as gb
    g = fixture()
    enclosed = [70 * nm, 70 * nm, 75 * nm]   # sphere, core + shell, the fixture's particle
    parts = [fixed_particle(g["position"][i], g["tmatrix"][i], enclosed[i]) for i in range(3)]
    c = gb.cluster(particles=parts, source=gb.plane_wave([1, 1j]), wavelength=float(g["wavelength"]), lmax=3,
                   medium=gb.constant_material(index=1.33), method=gb.solver.exact, **kw)
    return g, c


@pytest.mark.gpu
def test_cluster_matches_reference_cluster():
    g, c = _reference_cluster()
    assert c.solver_status == 0
    assert rel(c.p_src, g["p_src"]) < 1e-12
    assert rel(c.p_inc, g["p_inc"]) < 1e-10
    assert rel(c.p_scat, g["p_scat"]) < 1e-10
    C = c.cross_sections()
    np.testing.assert_allclose([C.scattering, C.absorption, C.extinction], g["cross_sections"], rtol=1e-9)
    per = np.array([[np.asarray(v) for v in c.cross_sections_per_multipole_of_particle(i)] for i in range(3)])
    assert rel(per, g["cross_sections_per_multipole"]) < 1e-9
    assert rel(c.force(), g["force"]) < 1e-9
    assert rel(c.torque(), g["torque"]) < 1e-9


@pytest.mark.gpu
def test_cluster_fields_match_reference_cluster():
    """E and H of the reference's cluster.E_field / H_field (cluster.py:219-345): the
    outgoing expansions plus the source outside, zero inside a particle's enclosed
    radius (interior=True or mask=True), 1e-9 of the largest field."""
    g, c = _reference_cluster()
    x, y, z = g["field_x"], g["field_y"], g["field_z"]
    assert rel(c.E_field(x, y, z), g["E_total"]) < 1e-9
    assert rel(c.H_field(x, y, z), g["H_total"]) < 1e-9
    assert rel(c.E_field(x, y, z, source=False, interior=False), g["E_scat_only"]) < 1e-9
    assert rel(c.E_field(x, y, z, mask=True), g["E_masked"]) < 1e-9


@pytest.mark.gpu
def test_cluster_coefficients_and_far_field_match_reference_cluster():
    """p_cluster (vsh/cluster_coefficients.py:14-53), the cluster cross-sections per
    multipole (cluster.py:379-391) and E/H_angular (cluster.py:349-377) of the
    reference's cluster: 1e-10 for the coefficients, 1e-8 for the far fields."""
    g, c = _reference_cluster()
    assert rel(c.solve_cluster_coefficients(), g["p_cluster"]) < 1e-10
    Cm = np.array([np.asarray(v) for v in c.cross_sections_per_multipole()])
    assert rel(Cm, g["cluster_xs_per_multipole"]) < 1e-9
    th, ph = g["far_theta"], g["far_phi"]
    assert rel(c.E_angular(th, ph), g["E_angular"]) < 1e-8
    assert rel(c.H_angular(th, ph), g["H_angular"]) < 1e-8


@pytest.mark.gpu
def test_cluster_mixed_precision_extinction():
    g, c = _reference_cluster(precision="mixed", tol=1e-10)
    assert c.solver_status == 0
    C = c.cross_sections()
    assert abs(C.extinction - g["cross_sections"][2]) / abs(g["cross_sections"][2]) < 1e-6
    assert rel(c.p_inc, g["p_inc"]) < 1e-7


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sphere_tmatrices_give_the_sphere_cluster(precision):
    """A cluster of spheres given as T-matrices is the sphere cluster (BiCGSTAB at
    the same tolerance on the same operator)."""
    import miepy_gb300 as gb
    pos, radius, eps, mie, k = random_cluster(11, N=16, lmax=4)
    wl = 620 * nm
    medium = gb.constant_material(index=1.33)
    mats = [gb.constant_material(eps=e) for e in eps]
    s = gb.sphere_cluster(position=pos, radius=radius, material=mats, source=gb.plane_wave([1, 0]), wavelength=wl,
                          lmax=4, medium=medium, precision=precision, tol=1e-11)
    parts = [gb.sphere(pos[i], radius[i], mats[i]) for i in range(len(pos))]
    t = gb.cluster(particles=parts, source=gb.plane_wave([1, 0]), wavelength=wl, lmax=4, medium=medium,
                   precision=precision, tol=1e-11)
    assert s.solver_status == 0 and t.solver_status == 0
    assert rel(t.p_inc, s.p_inc) < 1e-9
    assert rel(t.p_scat, s.p_scat) < 1e-9
    Cs, Ct = s.cross_sections(), t.cross_sections()
    np.testing.assert_allclose([Ct.scattering, Ct.absorption, Ct.extinction],
                               [Cs.scattering, Cs.absorption, Cs.extinction], rtol=1e-8)
    assert rel(t.force(), s.force()) < 1e-8
    assert rel(t.torque(), s.torque()) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tmatrix_batch_load_reuses_like_a_fresh_one(precision):
    from miepy_gb300 import ClusterBatch, plane_wave
    rng = np.random.default_rng(4)

    def spec(seed):
        pos, _, _, mie, k = random_cluster(seed, N=7, lmax=3)
        T = sphere_tmatrices(mie) + 0.01 * (rng.standard_normal((7, 2, 15, 2, 15))
                                            + 1j * rng.standard_normal((7, 2, 15, 2, 15)))
        return dict(position=pos, tmatrix=T, k=k, p_src=plane_wave([1, 0]).structure(pos, k, 3))

    a, b = spec(21), spec(22)
    reused = ClusterBatch([a], R=1, precision=precision)
    reused.assemble().solve(tol=1e-10, inner_tol=1e-4)
    reused.load([b])
    reused.assemble().solve(tol=1e-10, inner_tol=1e-4)
    reused.epilogue(1.33 ** 2)
    fresh = ClusterBatch([b], R=1, precision=precision).assemble()
    fresh.solve(tol=1e-10, inner_tol=1e-4)
    fresh.epilogue(1.33 ** 2)
    assert np.all(reused.status == 0) and np.all(fresh.status == 0)
    np.testing.assert_array_equal(reused.x.cpu().numpy(), fresh.x.cpu().numpy())
    np.testing.assert_array_equal(reused.xs.cpu().numpy(), fresh.xs.cpu().numpy())
    np.testing.assert_array_equal(reused.F.cpu().numpy(), fresh.F.cpu().numpy())
    with pytest.raises(ValueError):
        reused.load([dict(position=b["position"], mie_scat=np.zeros((7, 2, 3), complex), k=b["k"],
                          p_src=b["p_src"])])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,bound", [("fp64", 1e-11, 1e-9), ("mixed", 1e-11, 1e-8), ("fp32", 1e-5, 1e-3)])
def test_tmatrix_batch_of_clusters_with_two_rhs(precision, tol, bound):
    """Two clusters of different N and lmax in one batch, two right-hand sides each,
    dense random T-matrices: against the oracle's dense aggregate and an LU solve."""
    from miepy_gb300 import ClusterBatch, plane_wave
    from oracle import oracle as O
    rng = np.random.default_rng(9)
    specs = []
    for seed, N, lmax in [(31, 6, 3), (32, 9, 2)]:
        pos, _, _, mie, k = random_cluster(seed, N=N, lmax=lmax)
        rmax = lmax * (lmax + 2)
        shape = (N, 2, rmax, 2, rmax)
        T = sphere_tmatrices(mie) + 0.02 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
        p_src = np.stack([plane_wave([1, 0]).structure(pos, k, lmax), plane_wave([0, 1]).structure(pos, k, lmax)],
                         axis=-1)
        specs.append(dict(position=pos, tmatrix=T, k=k, p_src=p_src))
    b = ClusterBatch(specs, R=2, precision=precision).assemble()
    b.solve(tol=tol, inner_tol=1e-6)
    b.epilogue(1.33 ** 2)
    assert np.all(b.status == 0)
    for q, sp in enumerate(specs):
        A = O.particle_aggregate_tmatrix(sp["position"], sp["tmatrix"], sp["k"])
        D = A.shape[0]
        x_ref = np.linalg.solve(np.eye(D) + A, sp["p_src"].reshape(D, 2))
        x = b.cluster_view(q, b.x).cpu().numpy().reshape(D, 2)
        assert rel(x, x_ref) < bound
        p_scat = np.einsum("naibj,nbjr->nair", sp["tmatrix"], x_ref.reshape(sp["p_src"].shape))
        assert rel(b.cluster_view(q, b.p_scat).cpu().numpy(), p_scat) < bound


@pytest.mark.gpu
def test_cluster_without_interactions():
    """interactions=False: p_inc = p_src and p_scat = T p_src (cluster.py:648-650)."""
    import miepy_gb300 as gb
    g = fixture()
    parts = [fixed_particle(g["position"][i], g["tmatrix"][i]) for i in range(3)]
    c = gb.cluster(particles=parts, source=gb.plane_wave([1, 1j]), wavelength=float(g["wavelength"]), lmax=3,
                   medium=gb.constant_material(index=1.33), interactions=False)
    assert rel(c.p_inc, g["p_src"]) < 1e-12
    assert rel(c.p_scat, np.einsum("naibj,nbj->nai", g["tmatrix"], g["p_src"])) < 1e-12


def test_sphere_tmatrix_conducting_and_lossy_match_reference():
    """tmatrix_sphere (tmatrix/common.py:6-28) for a perfect conductor and a lossy
    dielectric in vacuum, against the reference's own T-matrices."""
    import miepy_gb300 as gb
    g = fixture()
    T = gb.tmatrix_sphere(60 * nm, 600 * nm, -10 + 1j, 1.33 ** 2, 3, conducting=True)
    assert rel(T, g["T_sphere_metal"]) < 1e-12
    T = gb.tmatrix_sphere(90 * nm, 700 * nm, 4.0 + 0.8j, 1.0, 3)
    assert rel(T, g["T_sphere_lossy"]) < 1e-12

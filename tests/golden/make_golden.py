"""Generate the golden fixtures in this directory.

Runs the reference's own Python layer (``miepy`` from the reference tree,
unmodified) on top of the CPU oracle registered as ``miepy.cpp``, and stores
inputs and outputs of the sphere-cluster path as small ``.npz`` files.  The GPU
parity tests compare the product against these fixtures without needing the
reference tree at run time.

Usage:  MIEPY_REFERENCE_SRC=/root/reference/src python tests/golden/make_golden.py [large | fields | beams | interior]
        (or with the reference staged by oracle/stage_reference.py:
         MIEPY_REFERENCE_SRC=baseline/_ref/src python tests/golden/make_golden.py [large | fields | beams | interior])
        MIEPY_REFERENCE_SRC=... python tests/golden/make_golden.py precond \
            /root/reference/benchmarks/results/final_performance_branch.json
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.refshim import import_reference  # noqa: E402

nm = 1e-9


def cluster_record(miepy, name, cluster, store_matrix=False, field_pts=None):
    c = cluster
    md = c.material_data
    rec = dict(
        position=c.position, radius=c.radius, wavelength=np.float64(c.wavelength), lmax=np.int64(c.lmax),
        eps=np.asarray(md.eps, complex), mu=np.asarray(md.mu, complex), n=np.asarray(md.n, complex),
        eps_b=np.complex128(md.eps_b), mu_b=np.complex128(md.mu_b), k_b=np.float64(np.real(md.k_b)),
        mie_scat=c.mie_scat, mie_int=c.mie_int, p_src=c.p_src, p_inc=c.p_inc, p_scat=c.p_scat, p_int=c.p_int,
    )
    C = c.cross_sections()
    rec["cross_sections"] = np.array([C.scattering, C.absorption, C.extinction], dtype=float)
    per = np.array([[np.asarray(v) for v in c.cross_sections_per_multipole_of_particle(i)]
                    for i in range(c.Nparticles)], dtype=float)   # [N, 3, 2, lmax]
    rec["cross_sections_per_multipole"] = per
    rec["force"] = c.force()
    rec["torque"] = c.torque()
    rec["force_nosource"] = c.force(source=False)
    # cluster coefficients about the origin and far fields (the f2 row)
    rec["p_cluster"] = miepy.cluster_coefficients(c.position, c.p_scat, md.k_b, origin=c.origin, lmax=c.lmax)
    rec["p_cluster_lmax_plus1"] = miepy.cluster_coefficients(c.position, c.p_scat, md.k_b, origin=c.origin,
                                                            lmax=min(c.lmax + 1, 8))
    Cm = c.cross_sections_per_multipole()
    rec["cluster_xs_per_multipole"] = np.array([np.asarray(v) for v in Cm], dtype=float)
    th_far = np.linspace(0.1, np.pi - 0.1, 5)
    ph_far = np.linspace(0.0, 2 * np.pi, 5)
    rec["far_theta"], rec["far_phi"] = th_far, ph_far
    rec["E_angular"] = c.E_angular(th_far, ph_far)
    rec["H_angular"] = c.H_angular(th_far, ph_far)
    if store_matrix:
        rec["agg_tmatrix"] = miepy.interactions.sphere_aggregate_tmatrix(c.position, c.mie_scat, md.k_b)
    if field_pts is not None:
        x, y, z = field_pts
        rec["field_x"], rec["field_y"], rec["field_z"] = x, y, z
        rec["E_total"] = c.E_field(x, y, z)
        rec["E_scat_only"] = c.E_field(x, y, z, source=False, interior=False)
        rec["H_total"] = c.H_field(x, y, z)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print("wrote", name, {k: np.shape(v) for k, v in rec.items() if np.ndim(v) > 1})


def random_positions(rng, N, rmin, rmax, box):
    pos, rad = [], []
    tries = 0
    while len(pos) < N:
        tries += 1
        if tries > 10**6:
            raise RuntimeError("rejection sampling failed")
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(0, box, size=3)
        if all(np.linalg.norm(c - p) > r + q for p, q in zip(pos, rad)):
            pos.append(c)
            rad.append(r)
    return np.array(pos), np.array(rad)


def main():
    miepy = import_reference()
    # dimer: radius 75 nm, n = 0.2+3.0i, centres (+-100 nm, 0, 0), water, x-polarised plane
    # wave along +z, 600 nm, lmax 6
    mat = miepy.constant_material(index=0.2 + 3.0j)
    water = miepy.materials.water()
    src_x = miepy.sources.plane_wave.from_string(polarization="x")
    pts = (np.array([0.0, 0.0, 150 * nm, -60 * nm, 300 * nm, 100 * nm]),
           np.array([0.0, 50 * nm, 0.0, 10 * nm, 200 * nm, 0.0]),
           np.array([0.0, 0.0, 40 * nm, 20 * nm, -100 * nm, 10 * nm]))
    kw = dict(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm, material=mat, source=src_x,
              wavelength=600 * nm, lmax=6, medium=water)
    cluster_record(miepy, "dimer_lmax6_exact", miepy.sphere_cluster(**kw, method=miepy.solver.exact),
                   store_matrix=True, field_pts=pts)
    cluster_record(miepy, "dimer_lmax6_bicgstab", miepy.sphere_cluster(**kw))
    # fields of one particle's expansions (sphere_cluster.py:150-200), at kr >= 10 from
    # particle 0 (the regular expansion's upward recurrence stays accurate there);
    # source=False last: the reference subtracts p_src from p_inc in place
    c = miepy.sphere_cluster(**kw, method=miepy.solver.exact)
    fx = np.array([700, -800, 100, 0.0, -500]) * nm
    fy = np.array([0.0, 300, 900, -850, 600]) * nm
    fz = np.array([200, -100, 50, 300, -400]) * nm
    rec = dict(field_x=fx, field_y=fy, field_z=fz, E0=c.E_field_from_particle(0, fx, fy, fz),
               H0=c.H_field_from_particle(0, fx, fy, fz), E1=c.E_field_from_particle(1, fx, fy, fz))
    rec["E0_nosource"] = c.E_field_from_particle(0, fx, fy, fz, source=False)
    np.savez_compressed(os.path.join(HERE, "dimer_lmax6_field_from_particle.npz"), **rec)
    print("wrote dimer_lmax6_field_from_particle")

    # five Ag spheres, rhc, lmax 2 (the reference's multi-particle BiCGSTAB case)
    Ag = miepy.materials.Ag()
    src_rhc = miepy.sources.plane_wave.from_string(polarization="rhc")
    five = [[0, 0, 0], [250 * nm, 0, 0], [-250 * nm, 0, 0], [0, 250 * nm, 0], [0, -250 * nm, 0]]
    for meth, tag in ((miepy.solver.exact, "exact"), (None, "bicgstab")):
        cluster_record(miepy, f"ag5_lmax2_{tag}",
                       miepy.sphere_cluster(position=five, radius=75 * nm, material=Ag, source=src_rhc,
                                            wavelength=600 * nm, lmax=2, method=meth),
                       store_matrix=(tag == "exact"))

    # random cluster: 12 spheres, radii 50-100 nm in a 1 um cube, n = 1.5+0.01i, lmax 3, vacuum,
    # y-polarised; and 6 spheres at lmax 8 (largest mode set)
    rng = np.random.default_rng(7)
    pos, rad = random_positions(rng, 12, 50 * nm, 100 * nm, 1000 * nm)
    diel = miepy.constant_material(index=1.5 + 0.01j)
    src_y = miepy.sources.plane_wave.from_string(polarization="y")
    cluster_record(miepy, "rand12_lmax3_exact",
                   miepy.sphere_cluster(position=pos, radius=rad, material=diel, source=src_y,
                                        wavelength=600 * nm, lmax=3, method=miepy.solver.exact),
                   field_pts=pts)
    pos, rad = random_positions(rng, 4, 50 * nm, 100 * nm, 800 * nm)
    cluster_record(miepy, "rand4_lmax8_exact",
                   miepy.sphere_cluster(position=pos, radius=rad, material=diel, source=src_x,
                                        wavelength=700 * nm, lmax=8, method=miepy.solver.exact))

    # Drude sphere pair (the wavelength-sweep material): eps = 9 - wp^2/(w^2 + i g w),
    # hbar wp = 9.0 eV, hbar g = 0.07 eV
    def drude(wav):
        w = 1239.84193e-9 / wav
        return 9.0 - 9.0**2 / (w**2 + 1j * 0.07 * w)

    dm = miepy.function_material(drude)
    for wav in (450 * nm, 800 * nm):
        cluster_record(miepy, f"drude2_lmax4_{int(round(wav / nm))}nm_exact",
                       miepy.sphere_cluster(position=[[0, 0, -90 * nm], [30 * nm, 20 * nm, 90 * nm]],
                                            radius=[60 * nm, 70 * nm], material=dm, source=src_x,
                                            wavelength=wav, lmax=4, method=miepy.solver.exact))

    # Gaussian beam (waist 1 um, x-polarised, vacuum, 600 nm): p_src at scattered
    # points (sources/beams.py:168-200) and a 3-sphere cluster driven by it
    beam = miepy.sources.gaussian_beam(width=1000 * nm, polarization=[1, 0])
    rng_b = np.random.default_rng(11)
    bpos = rng_b.uniform(-600 * nm, 600 * nm, size=(7, 3))
    k_v = 2 * np.pi / (600 * nm)
    rec = dict(position=bpos, k=np.float64(k_v), lmax=np.int64(5), width=np.float64(1000 * nm),
               polarization=np.array([1.0, 0.0]), p_src=beam.structure(bpos, k_v, 5),
               E0=np.float64(beam.E0(k_v)), theta_c=np.float64(beam.theta_cutoff(k_v)))
    np.savez_compressed(os.path.join(HERE, "gauss_beam_lmax5.npz"), **rec)
    print("wrote gauss_beam_lmax5")
    cluster_record(miepy, "gauss3_lmax3_exact",
                   miepy.sphere_cluster(position=[[0, 0, 0], [200 * nm, 50 * nm, 0], [-150 * nm, 100 * nm, 80 * nm]],
                                        radius=[70 * nm, 60 * nm, 80 * nm], material=diel,
                                        source=miepy.sources.gaussian_beam(width=1000 * nm, polarization=[1, 0]),
                                        wavelength=600 * nm, lmax=3, method=miepy.solver.exact),
                   store_matrix=True)

    # a trimer above a planar interface (substrate row): reflected source, reflection
    # matrix, solve, observables and fields with the reflected source
    sub = miepy.interface(miepy.constant_material(index=1.7), z=-120 * nm)
    c = miepy.sphere_cluster(position=[[0, 0, 0], [210 * nm, 40 * nm, 30 * nm], [-160 * nm, 90 * nm, 60 * nm]],
                             radius=[70 * nm, 60 * nm, 80 * nm], material=diel, medium=miepy.materials.water(),
                             source=miepy.sources.plane_wave([1, 0]), wavelength=600 * nm, lmax=3,
                             interface=sub, method=miepy.solver.exact)
    md = c.material_data
    r0 = sub.reflection_coefficients(theta=0, wavelength=c.wavelength, medium=c.medium)[0]
    C = c.cross_sections()
    fx = np.array([0.0, 300 * nm, -250 * nm, 50 * nm])
    fy = np.array([0.0, -100 * nm, 150 * nm, 400 * nm])
    fz = np.array([-60 * nm, 200 * nm, -40 * nm, 120 * nm])
    rec = dict(position=c.position, radius=c.radius, wavelength=np.float64(c.wavelength), lmax=np.int64(c.lmax),
               eps=np.asarray(md.eps, complex), n=np.asarray(md.n, complex), eps_b=np.complex128(md.eps_b),
               mu_b=np.complex128(md.mu_b), k_b=np.float64(np.real(md.k_b)), interface_z=np.float64(sub.z),
               interface_index=np.complex128(1.7), r0=np.complex128(r0), mie_scat=c.mie_scat, mie_int=c.mie_int,
               p_src=c.p_src, p_inc=c.p_inc, p_scat=c.p_scat, p_int=c.p_int,
               cross_sections=np.array([C.scattering, C.absorption, C.extinction], dtype=float),
               force=c.force(), torque=c.torque(),
               reflection_matrix=miepy.interactions.reflection_matrix_nia(c.position, c.mie_scat, md.k_b, r0, sub.z),
               field_x=fx, field_y=fy, field_z=fz, E_total=c.E_field(fx, fy, fz))
    np.savez_compressed(os.path.join(HERE, "interface3_lmax3_exact.npz"), **rec)
    print("wrote interface3_lmax3_exact")
    # the reference's interface identity (moving particle and interface together),
    # for a metallic sphere in water: both cross-section triples
    wat = miepy.constant_material(index=1.33)
    kw = dict(radius=75 * nm, material=miepy.constant_material(index=0.2 + 3.0j), medium=wat, lmax=2,
              wavelength=600 * nm, source=miepy.sources.plane_wave([1, 0]), method=miepy.solver.exact)
    c1 = miepy.sphere_cluster(position=[0, 0, -400 * nm], interface=miepy.interface(miepy.constant_material(index=1.7)),
                              **kw)
    c2 = miepy.sphere_cluster(position=[0, 0, 0],
                              interface=miepy.interface(miepy.constant_material(index=1.7), z=400 * nm), **kw)
    np.savez_compressed(os.path.join(HERE, "interface_identity.npz"), C1=np.array(c1.cross_sections()),
                        C2=np.array(c2.cross_sections()))
    print("wrote interface_identity")

    # general particles (T-matrix row): the reference's miepy.cluster with a sphere, a
    # core-shell particle and a particle whose T-matrix is a sphere's plus a dense
    # random part (every block non-diagonal), solved exactly
    rng = np.random.default_rng(20240611)
    lm = 3
    rm = lm * (lm + 2)
    base = miepy.tmatrix.tmatrix_sphere(65 * nm, 600 * nm, 3.2 + 0.1j, 1.33 ** 2, lm)
    T_dense = base + 0.15 * np.abs(base).max() * (rng.standard_normal((2, rm, 2, rm))
                                                  + 1j * rng.standard_normal((2, rm, 2, rm))) / np.sqrt(2 * rm)

    class fixed_tmatrix_particle(miepy.particles.particle_base.particle):
        def __init__(self, position, tmatrix):
            super().__init__(position, None, miepy.constant_material(index=1.8))
            self._T = tmatrix

        def compute_tmatrix(self, lmax, wavelength, eps_m, **kwargs):
            self.tmatrix = self.tmatrix_fixed = self._T
            return self._T

        def _dict_key(self, wavelength):
            return (fixed_tmatrix_particle, id(self))

        def enclosed_radius(self):
            return 75 * nm

    parts = [miepy.sphere([0, 0, 0], 70 * nm, miepy.constant_material(index=1.9 + 0.05j)),
             miepy.core_shell([220 * nm, 30 * nm, -40 * nm], 50 * nm, 20 * nm, miepy.constant_material(index=0.3 + 3j),
                              miepy.constant_material(index=1.5)),
             fixed_tmatrix_particle([-150 * nm, 120 * nm, 70 * nm], T_dense)]
    c = miepy.cluster(particles=parts, source=miepy.sources.plane_wave([1, 1j]), wavelength=600 * nm, lmax=lm,
                      medium=miepy.constant_material(index=1.33), method=miepy.solver.exact)
    # field points: outside every particle, plus one inside the sphere and one inside
    # the core-shell particle (interior rule)
    fx = np.array([0.0, 300 * nm, -250 * nm, 50 * nm, 10 * nm, 225 * nm])
    fy = np.array([0.0, -100 * nm, 150 * nm, 400 * nm, 5 * nm, 35 * nm])
    fz = np.array([-200 * nm, 200 * nm, -40 * nm, 120 * nm, 0.0, -40 * nm])
    md = c.material_data
    C = c.cross_sections()
    per = np.array([[np.asarray(v) for v in c.cross_sections_per_multipole_of_particle(i)]
                    for i in range(c.Nparticles)], dtype=float)
    np.savez_compressed(os.path.join(HERE, "tmatrix3_lmax3_exact.npz"), position=c.position, tmatrix=c.tmatrix,
                        wavelength=np.float64(c.wavelength), lmax=np.int64(lm), eps_b=np.complex128(md.eps_b),
                        mu_b=np.complex128(md.mu_b), k_b=np.float64(np.real(md.k_b)), p_src=c.p_src, p_inc=c.p_inc,
                        p_scat=c.p_scat, cross_sections=np.array([C.scattering, C.absorption, C.extinction]),
                        cross_sections_per_multipole=per, force=c.force(), torque=c.torque(),
                        agg_tmatrix=miepy.interactions.particle_aggregate_tmatrix(c.position, c.tmatrix, md.k_b),
                        field_x=fx, field_y=fy, field_z=fz, E_total=c.E_field(fx, fy, fz), H_total=c.H_field(fx, fy, fz),
                        E_scat_only=c.E_field(fx, fy, fz, source=False, interior=False),
                        E_masked=c.E_field(fx, fy, fz, mask=True),
                        p_cluster=miepy.cluster_coefficients(c.position, c.p_scat, md.k_b, origin=c.origin, lmax=lm),
                        cluster_xs_per_multipole=np.array([np.asarray(v) for v in c.cross_sections_per_multipole()]),
                        far_theta=np.linspace(0.1, np.pi - 0.1, 5), far_phi=np.linspace(0.0, 2 * np.pi, 5),
                        E_angular=c.E_angular(np.linspace(0.1, np.pi - 0.1, 5), np.linspace(0.0, 2 * np.pi, 5)),
                        H_angular=c.H_angular(np.linspace(0.1, np.pi - 0.1, 5), np.linspace(0.0, 2 * np.pi, 5)),
                        T_sphere_metal=miepy.tmatrix.tmatrix_sphere(60 * nm, 600 * nm, -10 + 1j, 1.33 ** 2, lm,
                                                                    conducting=True),
                        T_sphere_lossy=miepy.tmatrix.tmatrix_sphere(90 * nm, 700 * nm, 4.0 + 0.8j, 1.0, lm))
    print("wrote tmatrix3_lmax3_exact")

    # periodic clusters (lattice row): the reference's own lattice sums
    # (interactions.sphere_aggregate_tmatrix_periodic over symmetry.generate(5000))
    # and sphere_cluster(symmetry=...) solves: a dimer in a square lattice under an
    # oblique plane wave, and one sphere in a chain along x
    for name, sym, pos, rad, lm, src in [
            ("periodic_square_dimer_lmax2", miepy.symmetry.square_lattice_2d(700 * nm),
             [[-120 * nm, 20 * nm, 0], [130 * nm, -40 * nm, 30 * nm]], [70 * nm, 60 * nm], 2,
             miepy.sources.plane_wave([1, 0.5j], theta=0.35, phi=0.6)),
            ("periodic_chain_single_lmax3", miepy.symmetry.x_translation_1d(450 * nm), [[0, 0, 0]], [80 * nm], 3,
             miepy.sources.plane_wave([0, 1], theta=0.5, phi=0.0))]:
        c = miepy.sphere_cluster(position=pos, radius=rad, material=miepy.constant_material(index=1.8 + 0.02j),
                                 medium=miepy.constant_material(index=1.33), source=src, wavelength=620 * nm, lmax=lm,
                                 symmetry=sym, method=miepy.solver.exact)
        md = c.material_data
        xs_, ys_, zs_ = sym.generate(5000)
        C = c.cross_sections()
        agg = miepy.interactions.sphere_aggregate_tmatrix_periodic(c.position, c.mie_scat, md.k_b, sym,
                                                                   src.k_hat)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), position=c.position, radius=c.radius,
                            wavelength=np.float64(c.wavelength), lmax=np.int64(lm), k_b=np.float64(np.real(md.k_b)),
                            eps=np.asarray(md.eps, complex), k_hat=np.asarray(src.k_hat, float),
                            cells=np.array([xs_, ys_, zs_]).T, mie_scat=c.mie_scat, mie_int=c.mie_int, p_src=c.p_src,
                            p_inc=c.p_inc, p_scat=c.p_scat, p_int=c.p_int, agg_tmatrix=agg,
                            cross_sections=np.array([C.scattering, C.absorption, C.extinction]), force=c.force(),
                            torque=c.torque())
        print("wrote", name)

    # a periodic dimer above an interface: the lattice sums minus the reflection
    # matrix (sphere_cluster.py:694-710 with both options)
    sym = miepy.symmetry.square_lattice_2d(650 * nm)
    sub = miepy.interface(miepy.constant_material(index=1.6), z=-150 * nm)
    c = miepy.sphere_cluster(position=[[-100 * nm, 0, 0], [120 * nm, 30 * nm, 20 * nm]], radius=[70 * nm, 60 * nm],
                             material=miepy.constant_material(index=2.0 + 0.05j),
                             medium=miepy.constant_material(index=1.33), source=miepy.sources.plane_wave([1, 0]),
                             wavelength=640 * nm, lmax=2, symmetry=sym, interface=sub, method=miepy.solver.exact)
    C = c.cross_sections()
    np.savez_compressed(os.path.join(HERE, "periodic_interface_dimer_lmax2.npz"), position=c.position,
                        radius=c.radius, wavelength=np.float64(c.wavelength), p_src=c.p_src, p_inc=c.p_inc,
                        p_scat=c.p_scat, cross_sections=np.array([C.scattering, C.absorption, C.extinction]),
                        force=c.force(), torque=c.torque())
    print("wrote periodic_interface_dimer_lmax2")

    # special-function tables for the device recurrences
    from oracle import oracle as O
    z = np.linspace(-0.999, 0.999, 23)
    leg = np.array([O.associated_legendre_recursion(17, zz) for zz in z])
    x = np.linspace(0.05, 40.0, 29)
    hn = np.array([O.spherical_hn_recursion(17, xx) for xx in x])
    np.savez_compressed(os.path.join(HERE, "special_tables.npz"), legendre_z=z, legendre=leg, hn_x=x, hn=hn)
    print("wrote special_tables")


def _observables(c):
    """p coefficients, cross-sections (total and per particle per multipole), force
    and torque of a solved reference cluster."""
    C = c.cross_sections()
    return dict(
        p_src=c.p_src, p_inc=c.p_inc, p_scat=c.p_scat, p_int=c.p_int,
        cross_sections=np.array([C.scattering, C.absorption, C.extinction], dtype=float),
        cross_sections_per_multipole=np.array([[np.asarray(v) for v in c.cross_sections_per_multipole_of_particle(i)]
                                               for i in range(c.Nparticles)], dtype=float),
        force=c.force(), torque=c.torque())


def _lapack_exact(miepy):
    """Route the exact solve (method=solver.exact) of the oracle standing in for
    miepy.cpp to LAPACK's partial-pivot LU (numpy.linalg.solve): the same algorithm
    class as the reference's Eigen partialPivLu, multithreaded, so that systems of
    D = 10^4 - 3 10^4 solve in seconds to minutes.  (I + T) is formed in place on
    the reference's aggregate and restored afterwards."""
    interactions = sys.modules["miepy.cpp.interactions"]
    plain = interactions.solve_linear_system

    def solve(agg, p_src, method=None, *a, **k):
        if getattr(method, "name", method) != "exact":
            return plain(agg, p_src, method, *a, **k)
        D = p_src.size
        A = agg.reshape(D, D)
        A[np.diag_indices(D)] += 1.0
        try:
            return np.linalg.solve(A, p_src.reshape(D))
        finally:
            A[np.diag_indices(D)] -= 1.0

    interactions.solve_linear_system = solve
    return plain


def large_main():
    """Fixtures at the benchmark's own sizes (exact solves, LAPACK LU):

    config2_n200_lmax4_exact  N = 200 spheres, radii U[50, 100] nm in a 2 um cube
        (rejection sampling, seed 2: the benchmark's cluster), n = 1.5+0.01i, vacuum,
        600 nm, lmax 4 (D = 9600); x- and y-polarised plane waves along +z;
    sweep_n100_lmax7_400nm_exact  the wavelength sweep's cluster (N = 100 Drude
        spheres, radii U[40, 80] nm, seed 3) at its first wavelength, 400 nm, where
        the adaptive rule gives lmax 7 (D = 12600);
    serve_n300_lmax6_exact  a serving-size request: N = 300 spheres, radii
        U[50, 100] nm in a centred cube of side (N (0.5 um)^3)^(1/3) (rejection
        sampling, seed 404), n = 1.9+0.05i, vacuum, 600 nm, lmax 6 (D = 28800),
        x-polarised plane wave.
    """
    miepy = import_reference()
    _lapack_exact(miepy)
    exact = miepy.solver.exact

    rng = np.random.default_rng(2)
    pos, rad = random_positions(rng, 200, 50 * nm, 100 * nm, 2000 * nm)
    diel = miepy.constant_material(index=1.5 + 0.01j)
    rec = dict(position=pos, radius=rad, wavelength=np.float64(600 * nm), lmax=np.int64(4))
    for pol in ("x", "y"):
        c = miepy.sphere_cluster(position=pos, radius=rad, material=diel,
                                 source=miepy.sources.plane_wave.from_string(polarization=pol),
                                 wavelength=600 * nm, lmax=4, method=exact)
        rec["k_b"] = np.float64(np.real(c.material_data.k_b))
        rec["mie_scat"], rec["mie_int"] = c.mie_scat, c.mie_int
        rec.update({f"{k}_{pol}": v for k, v in _observables(c).items()})
    np.savez_compressed(os.path.join(HERE, "config2_n200_lmax4_exact.npz"), **rec)
    print("wrote config2_n200_lmax4_exact")

    def drude(wav):
        w = 1239.84193e-9 / wav
        return 9.0 - 9.0**2 / (w**2 + 1j * 0.07 * w)

    rng = np.random.default_rng(3)
    pos, rad = random_positions(rng, 100, 40 * nm, 80 * nm, 2000 * nm)
    c = miepy.sphere_cluster(position=pos, radius=rad, material=miepy.function_material(drude),
                             source=miepy.sources.plane_wave.from_string(polarization="x"),
                             wavelength=400 * nm, lmax=7, method=exact)
    rec = dict(position=pos, radius=rad, wavelength=np.float64(400 * nm), lmax=np.int64(7),
               k_b=np.float64(np.real(c.material_data.k_b)), eps=np.asarray(c.material_data.eps, complex),
               mie_scat=c.mie_scat, mie_int=c.mie_int, **_observables(c))
    np.savez_compressed(os.path.join(HERE, "sweep_n100_lmax7_400nm_exact.npz"), **rec)
    print("wrote sweep_n100_lmax7_400nm_exact")

    rng = np.random.default_rng(404)
    N = 300
    side = (N * (500 * nm) ** 3) ** (1 / 3)
    pos, rad = random_positions(rng, N, 50 * nm, 100 * nm, side)
    pos = pos - side / 2
    c = miepy.sphere_cluster(position=pos, radius=rad, material=miepy.constant_material(index=1.9 + 0.05j),
                             source=miepy.sources.plane_wave.from_string(polarization="x"),
                             wavelength=600 * nm, lmax=6, method=exact)
    rec = dict(position=pos, radius=rad, wavelength=np.float64(600 * nm), lmax=np.int64(6),
               k_b=np.float64(np.real(c.material_data.k_b)), mie_scat=c.mie_scat, mie_int=c.mie_int,
               **_observables(c))
    np.savez_compressed(os.path.join(HERE, "serve_n300_lmax6_exact.npz"), **rec)
    print("wrote serve_n300_lmax6_exact")


def beams_main():
    """Rotated and reflected Gaussian beams (the reference's rotation runs with the
    harness's stand-in for the ``spherical`` package's Wigner-D matrices):
    gauss_beam_rotated_lmax5  p_src of beams (waist 1 um, 600 nm, vacuum) at
        (theta, phi) = (0.6, 0.9) centred off the origin, (pi, 0) and (1.2, -2.0)
        with circular polarisation, at 7 positions, lmax 5;
    interface_gauss3_lmax3_exact  the substrate trimer of interface3_lmax3_exact
        driven by a Gaussian beam (waist 1 um): p_src with the reflected beam, p_inc,
        cross-sections, forces and torques."""
    miepy = import_reference()
    k_v = 2 * np.pi / (600 * nm)
    rng_b = np.random.default_rng(12)
    bpos = rng_b.uniform(-600 * nm, 600 * nm, size=(7, 3))
    specs = [dict(theta=0.6, phi=0.9, polarization=[1, 0], center=[50 * nm, -30 * nm, 20 * nm]),
             dict(theta=np.pi, phi=0.0, polarization=[0, 1], center=[0, 0, 0]),
             dict(theta=1.2, phi=-2.0, polarization=[1, 1j], center=[-40 * nm, 0, 70 * nm])]
    rec = dict(position=bpos, k=np.float64(k_v), lmax=np.int64(5), width=np.float64(1000 * nm))
    for q, sp in enumerate(specs):
        b = miepy.sources.gaussian_beam(width=1000 * nm, polarization=sp["polarization"], theta=sp["theta"],
                                        phi=sp["phi"], center=sp["center"])
        rec[f"theta_{q}"], rec[f"phi_{q}"] = np.float64(sp["theta"]), np.float64(sp["phi"])
        rec[f"polarization_{q}"] = np.asarray(sp["polarization"], complex)
        rec[f"center_{q}"] = np.asarray(sp["center"], float)
        rec[f"p_src_{q}"] = b.structure(bpos, k_v, 5)
    np.savez_compressed(os.path.join(HERE, "gauss_beam_rotated_lmax5.npz"), **rec)
    print("wrote gauss_beam_rotated_lmax5")
    sub = miepy.interface(miepy.constant_material(index=1.7), z=-120 * nm)
    c = miepy.sphere_cluster(position=[[0, 0, 0], [210 * nm, 40 * nm, 30 * nm], [-160 * nm, 90 * nm, 60 * nm]],
                             radius=[70 * nm, 60 * nm, 80 * nm], material=miepy.constant_material(index=1.5 + 0.01j),
                             medium=miepy.materials.water(),
                             source=miepy.sources.gaussian_beam(width=1000 * nm, polarization=[1, 0]),
                             wavelength=600 * nm, lmax=3, interface=sub, method=miepy.solver.exact)
    C = c.cross_sections()
    rec = dict(position=c.position, radius=c.radius, p_src=c.p_src, p_inc=c.p_inc, p_scat=c.p_scat,
               cross_sections=np.array([C.scattering, C.absorption, C.extinction], dtype=float),
               force=c.force(), torque=c.torque())
    np.savez_compressed(os.path.join(HERE, "interface_gauss3_lmax3_exact.npz"), **rec)
    print("wrote interface_gauss3_lmax3_exact")


def fields_main():
    """Far-field and spherical-coordinate fields of the water dimer (lmax 6, exact
    solve): E and H with far=True (Cartesian points 50 um away, and the same points
    given as (r, theta, phi) with spherical=True) and near fields with
    spherical=True at r = 400 nm about the origin."""
    miepy = import_reference()
    c = miepy.sphere_cluster(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
                             material=miepy.constant_material(index=0.2 + 3.0j),
                             source=miepy.sources.plane_wave.from_string(polarization="x"),
                             wavelength=600 * nm, lmax=6, medium=miepy.materials.water(), method=miepy.solver.exact)
    th = np.linspace(0.2, np.pi - 0.2, 5)
    ph = np.linspace(0.1, 2 * np.pi - 0.3, 5)
    r_far = np.full(5, 50e-6)
    r_near = np.full(5, 400 * nm)
    x, y, z = miepy.coordinates.sph_to_cart(r_far, th, ph)
    rec = dict(theta=th, phi=ph, r_far=r_far, r_near=r_near, x_far=x, y_far=y, z_far=z,
               E_far=c.E_field(x, y, z, far=True), H_far=c.H_field(x, y, z, far=True),
               E_far_sph=c.E_field(r_far, th, ph, far=True, spherical=True),
               H_far_sph=c.H_field(r_far, th, ph, far=True, spherical=True),
               E_far_scat_sph=c.E_field(r_far, th, ph, far=True, spherical=True, source=False),
               E_near_sph=c.E_field(r_near, th, ph, spherical=True),
               H_near_sph=c.H_field(r_near, th, ph, spherical=True))
    np.savez_compressed(os.path.join(HERE, "dimer_lmax6_far_spherical.npz"), **rec)
    print("wrote dimer_lmax6_far_spherical")


def _mp_spherical_jn(n, z, derivative=False, dps=40):
    """j_n(z) (or j_n'(z)) of complex z at dps digits (mpmath Bessel J of order
    n + 1/2), rounded to complex128; arrays elementwise."""
    import mpmath
    mpmath.mp.dps = dps
    zz = np.asarray(z, dtype=complex)
    out = np.empty(zz.shape, dtype=complex)

    def jn(order, w):
        if order < 0:   # j_{-1}(w) = cos(w) / w
            return mpmath.cos(w) / w
        return mpmath.sqrt(mpmath.pi / (2 * w)) * mpmath.besselj(order + mpmath.mpf(1) / 2, w)

    for idx, v in np.ndenumerate(zz):
        w = mpmath.mpc(v.real, v.imag)
        val = jn(n - 1, w) - (n + 1) / w * jn(n, w) if derivative else jn(n, w)
        out[idx] = complex(val)
    return out


def interior_main():
    """Interior fields against high-precision j_n:
    interior_dimer_lmax6  the dimer of dimer_lmax6_exact (index 0.2 + 3i in water,
        |k_int r| < 2.4), 40 points inside each sphere at 0.5 .. 74 nm from its
        centre, and 8 outside;
    interior_big_lmax8  two dielectric spheres (index 4 + 0.01i, radius 300 nm,
        600 nm, vacuum, lmax 8, |k_int r| up to 12.6), 40 points inside each.
    Each holds E and H from the reference as it is (j_n by the upward recurrence
    of cpp/src/special.cpp:20-45, as restated by the oracle) and from the reference
    with spherical_jn replaced by a 40-digit mpmath evaluation."""
    miepy = import_reference()
    rng = np.random.default_rng(31)

    def points(centres, radius, per, r_lo):
        out = []
        for c in centres:
            r = np.exp(rng.uniform(np.log(r_lo), np.log(0.99 * radius), per))
            u = rng.normal(size=(per, 3))
            u /= np.linalg.norm(u, axis=1)[:, None]
            out.append(np.asarray(c)[None, :] + r[:, None] * u)
        return np.concatenate(out)

    cases = dict(
        interior_dimer_lmax6=dict(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
                                  material=miepy.constant_material(index=0.2 + 3.0j), medium=miepy.materials.water(),
                                  lmax=6, r_lo=0.5 * nm, outside=8),
        interior_big_lmax8=dict(position=[[-350 * nm, 0, 0], [350 * nm, 0, 0]], radius=300 * nm,
                                material=miepy.constant_material(index=4.0 + 0.01j), medium=None,
                                lmax=8, r_lo=2 * nm, outside=0))
    for name, cs in cases.items():
        kw = dict(position=cs["position"], radius=cs["radius"], material=cs["material"],
                  source=miepy.sources.plane_wave.from_string(polarization="x"), wavelength=600 * nm,
                  lmax=cs["lmax"], method=miepy.solver.exact)
        if cs["medium"] is not None:
            kw["medium"] = cs["medium"]
        c = miepy.sphere_cluster(**kw)
        pts = points(cs["position"], cs["radius"], 40, cs["r_lo"])
        if cs["outside"]:
            pts = np.concatenate([pts, rng.uniform(-300 * nm, 300 * nm, size=(cs["outside"], 3)) + [0, 200 * nm, 0]])
        x, y, z = pts.T
        rec = dict(position=c.position, radius=c.radius, lmax=np.int64(cs["lmax"]), field_x=x, field_y=y, field_z=z,
                   E_ref=c.E_field(x, y, z), H_ref=c.H_field(x, y, z))
        saved = miepy.vsh.special.spherical_jn
        miepy.vsh.special.spherical_jn = _mp_spherical_jn
        try:
            rec["E_mp"], rec["H_mp"] = c.E_field(x, y, z), c.H_field(x, y, z)
        finally:
            miepy.vsh.special.spherical_jn = saved
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
        print("wrote", name)


def precond_main(results_json):
    """Linear chains of silver spheres (radius 75 nm, 600 nm, rhc plane wave) of the
    reference's solver benchmark (benchmarks/bench_solver.py:40-115), at the 15
    (N, lmax, separation) points of its committed results file (passed as the
    argument): positions, Mie coefficients, k and p_src from the reference, the
    diagonal of its build_block_preconditioner_sphere, and the numbers the results
    file holds for them (iterations, residuals, Frobenius norm of I + T, relative
    difference of the two solutions) from its bicgstab_profiled and
    bicgstab_preconditioned_profiled."""
    import json
    miepy = import_reference()
    with open(results_json) as f:
        data = json.load(f)
    ents = []

    def walk(o):
        if isinstance(o, dict):
            if "iterations_preconditioned" in o:
                ents.append(o)
            for v in o.values():
                walk(v)
        elif isinstance(o, list):
            for v in o:
                walk(v)

    walk(data)
    rec = dict(count=np.int64(len(ents)))
    keys = ("iterations", "residual", "iterations_preconditioned", "residual_preconditioned", "frobenius_norm",
            "solution_relative_diff")
    for q, e in enumerate(ents):
        N, lmax, sf = int(e["N"]), int(e["lmax"]), float(e["sep_factor"])
        pos = np.zeros((N, 3))
        pos[:, 0] = np.arange(N) * sf * 2 * 75 * nm
        c = miepy.sphere_cluster(position=pos, radius=75 * nm, material=miepy.materials.Ag(),
                                 source=miepy.sources.plane_wave.from_string(polarization="rhc"),
                                 wavelength=600 * nm, lmax=lmax)
        M, bs = miepy.interactions.build_block_preconditioner_sphere(c.mie_scat, lmax)
        rows = np.arange(M.shape[0])
        rec[f"N_{q}"], rec[f"lmax_{q}"], rec[f"sep_factor_{q}"] = np.int64(N), np.int64(lmax), np.float64(sf)
        rec[f"position_{q}"] = c.position
        rec[f"mie_scat_{q}"] = c.mie_scat
        rec[f"k_b_{q}"] = np.float64(np.real(c.material_data.k_b))
        rec[f"p_src_{q}"] = c.p_src
        rec[f"pdiag_{q}"] = M[rows, rows % bs]
        rec[f"expected_{q}"] = np.array([float(e[k]) for k in keys])
    rec["expected_keys"] = np.array(keys)
    np.savez_compressed(os.path.join(HERE, "precond_ag_chains.npz"), **rec)
    print("wrote precond_ag_chains")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "interior":
        interior_main()
    elif len(sys.argv) > 2 and sys.argv[1] == "precond":
        precond_main(sys.argv[2])
    elif len(sys.argv) > 1 and sys.argv[1] == "large":
        large_main()
    elif len(sys.argv) > 1 and sys.argv[1] == "fields":
        fields_main()
    elif len(sys.argv) > 1 and sys.argv[1] == "beams":
        beams_main()
    else:
        main()

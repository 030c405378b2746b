"""GPU parity tests: the CUDA path against the oracle and the golden fixtures.

Tolerances (stated per assertion): translation tables and assembled matrices
1e-12 relative to the largest entry; FP64 solves against the exact solution
1e-10 (p coefficients) and 1e-9 (cross-sections, forces, torques); BiCGSTAB at
the reference's tolerance against the reference's own BiCGSTAB result 1e-4 (the
reference's own GPU-vs-CPU bar); complex64 products 2e-6; mixed precision
C_ext within 1e-6 of FP64.
"""

import ctypes

import numpy as np
import pytest
import torch

import miepy_gb300 as gb
from miepy_gb300 import _native as nat
from miepy_gb300.engine import ClusterBatch, current_stream
from oracle import oracle as O
from tests import _golden as G

pytestmark = pytest.mark.gpu

nm = 1e-9


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(np.asarray(b))), 1e-300))


def batch_from_golden(g, precision="fp64", R=1):
    return ClusterBatch([dict(position=g["position"], mie_scat=g["mie_scat"], mie_int=g["mie_int"], k=float(g["k_b"]),
                              p_src=g["p_src"])], R=R, precision=precision)


def random_cluster(rng, N, rmin, rmax_, box):
    pos, rad = [], []
    while len(pos) < N:
        r = rng.uniform(rmin, rmax_)
        c = rng.uniform(0, box, size=3)
        if all(np.linalg.norm(c - p) > r + q for p, q in zip(pos, rad)):
            pos.append(c)
            rad.append(r)
    return np.array(pos), np.array(rad)


# ------------------------------------------------------------------ tables --
@pytest.mark.parametrize("lmax", [1, 2, 4, 6, 8, 10])
def test_translation_tables_match_oracle_cache(lmax):
    L = nat.lib()
    M = ctypes.c_int(0)
    assert L.gb_tables_count(lmax, ctypes.byref(M)) == 0
    M = M.value
    Q = lmax + 1
    nmvu = np.zeros((M, 4), np.int32)
    qab = np.zeros((M, 2), np.int32)
    cA = np.zeros((M, Q))
    cB = np.zeros((M, Q))
    nat.check(L.gb_tables_export(lmax, nmvu.ctypes.data, qab.ctypes.data, cA.ctypes.data, cB.ctypes.data, None))
    worst = 0.0
    gA = gB = 0.0
    for t in range(M):
        n, m, v, u = nmvu[t]
        factor, qa, qb, A, B = O.vsh_cache_entry(n, -m, v, u)
        gA = max(gA, np.max(np.abs(factor * A)))
        gB = max(gB, np.max(np.abs(factor * B)))
    for t in range(M):
        n, m, v, u = nmvu[t]
        factor, qa, qb, A, B = O.vsh_cache_entry(n, -m, v, u)
        assert (qa, qb) == tuple(qab[t])
        ia = (1j) ** (n + v)
        expA = np.real(factor * A / ia)
        expB = np.real(-factor * B[1:] / (ia * 1j))
        # relative to the entry, with an absolute floor at 1e-13 of the table's scale
        errA = np.abs(cA[t, : qa + 1] - expA) / np.maximum(np.abs(expA), 1e-3 * gA)
        worst = max(worst, np.max(errA))
        if qb >= 1:
            errB = np.abs(cB[t, 1: qb + 1] - expB) / np.maximum(np.abs(expB), 1e-3 * gB)
            worst = max(worst, np.max(errB))
    assert worst < 1e-10, worst


# --------------------------------------------------------------- assembly --
def dense_on_device(pos, mie, k, lmax):
    dev = torch.device("cuda")
    N = pos.shape[0]
    D = 2 * lmax * (lmax + 2) * N
    P = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
    Mi = torch.from_numpy(np.ascontiguousarray(mie)).to(dev)
    out = torch.empty((D, D), dtype=torch.complex128, device=dev)
    nat.check(nat.lib().gb_assemble_sphere_dense(N, lmax, nat.ptr(P), nat.ptr(Mi), float(k), nat.ptr(out),
                                                 current_stream()))
    return out.cpu().numpy()


@pytest.mark.parametrize("name", ["dimer_lmax6_exact", "ag5_lmax2_exact"])
def test_dense_assembly_matches_reference(name):
    g = G.load(name)
    T = dense_on_device(g["position"], g["mie_scat"], g["k_b"], int(g["lmax"]))
    ref = g["agg_tmatrix"].reshape(T.shape)
    assert rel(T, ref) < 1e-12


@pytest.mark.parametrize("N,lmax,seed", [(7, 3, 1), (4, 8, 2), (12, 1, 3), (9, 5, 4), (3, 9, 5), (3, 10, 6)])
def test_dense_assembly_matches_oracle_random(N, lmax, seed):
    rng = np.random.default_rng(seed)
    pos, _ = random_cluster(rng, N, 50 * nm, 90 * nm, 1200 * nm)
    mie = rng.normal(size=(N, 2, lmax)) + 1j * rng.normal(size=(N, 2, lmax))
    k = 2 * np.pi / (600 * nm)
    T = dense_on_device(pos, mie, k, lmax)
    ref = O.sphere_aggregate_tmatrix(pos, mie.reshape(N, -1), k)
    # lmax 9 and 10: the Gaunt coefficients of orders up to 20 and the Hankel and
    # Legendre recurrences to order 21 part between the two sides' methods by more
    # than at lmax <= 8; held to the translation tables' own 1e-10
    assert rel(T, ref) < (1e-12 if lmax <= 8 else 1e-10)


@pytest.mark.parametrize("N,lmax,R", [(6, 3, 1), (5, 4, 2), (3, 8, 2), (25, 2, 1), (40, 3, 2)])
def test_packed_operator_matches_oracle_matvec(N, lmax, R):
    rng = np.random.default_rng(N * 10 + lmax)
    pos, _ = random_cluster(rng, N, 40 * nm, 80 * nm, 1500 * nm)
    mie = (rng.normal(size=(N, 2, lmax)) + 1j * rng.normal(size=(N, 2, lmax))) * 0.3
    k = 2 * np.pi / (650 * nm)
    rmax = lmax * (lmax + 2)
    x = rng.normal(size=(N, 2, rmax, R)) + 1j * rng.normal(size=(N, 2, rmax, R))
    T = O.sphere_aggregate_tmatrix(pos, mie.reshape(N, -1), k)
    D = T.shape[0]
    ref = np.stack([O.gemv(T, x.reshape(D, R)[:, r]) + x.reshape(D, R)[:, r] for r in range(R)], axis=1)
    b = ClusterBatch([dict(position=pos, mie_scat=mie, k=k, p_src=x)], R=R, precision="fp64").assemble()
    bm = ClusterBatch([dict(position=pos, mie_scat=mie, k=k, p_src=x)], R=R, precision="mixed").assemble()
    xd = torch.from_numpy(x.reshape(-1)).to(b.device)
    y128 = b.apply(xd, "fp64").cpu().numpy().reshape(D, R)
    y64 = bm.apply(xd, "fp32").cpu().numpy().reshape(D, R)
    ydf = bm.apply(xd, "mixed").cpu().numpy().reshape(D, R)
    assert rel(y128, ref) < 1e-12      # FP64 arithmetic
    assert rel(y64, ref) < 2e-6        # complex64 matrix and arithmetic
    assert rel(ydf, ref) < 1e-12       # double-float hi + lo


def test_double_float_planes_match_fp64_blocks():
    """The mixed path's hi + lo planes (G tables from the special-function pass,
    tuple sums in double-float) against the FP64 path's complex128 blocks, in one
    ragged batch over lmax 1..10 (at lmax 10 both paths form the A and B sums in two
    passes): 1e-12 relative to each block's largest entry."""
    rng = np.random.default_rng(7)
    shapes = [(5, 1), (7, 2), (12, 3), (30, 4), (9, 4), (9, 5), (5, 6), (4, 7), (4, 8), (3, 9), (3, 10)]
    specs = []
    for N, lmax in shapes:
        pos, _ = random_cluster(rng, N, 40 * nm, 80 * nm, 1500 * nm)
        rmax = lmax * (lmax + 2)
        specs.append(dict(position=pos, mie_scat=np.ones((N, 2, lmax), complex), k=2 * np.pi / (rng.uniform(450, 900) * nm),
                          p_src=np.ones((N, 2, rmax, 1), complex)))
    b = ClusterBatch(specs, R=1, precision="fp64").assemble()
    bm = ClusterBatch(specs, R=1, precision="mixed").assemble()
    torch.cuda.synchronize()
    m128 = b.mat128.cpu().numpy()
    mdf = bm.mat64.cpu().numpy().astype(np.complex128) + bm.mat64lo.cpu().numpy().astype(np.complex128)
    for lay, lay_m in zip(b.layout, bm.layout):
        N, B = lay["N"], 2 * lay["rmax"]
        P = N * (N - 1) // 2
        ref = m128[lay["mat_off"]: lay["mat_off"] + P * B * B].reshape(P, B * B)
        got = mdf[lay_m["mat_off"]: lay_m["mat_off"] + P * B * B].reshape(P, B * B)
        err = np.max(np.abs(got - ref), axis=1) / np.max(np.abs(ref), axis=1)
        assert err.max() < 1e-12, (N, lay["lmax"], err.max())


def test_packed_assembly_at_odd_offsets():
    """The packed double-float assembly through gb_assemble_batch with the clusters'
    blocks at odd element offsets (8-byte aligned, so the block writes take the
    one-element path) equals the same assembly at aligned offsets, bit for bit, at
    lmax 4 and 5 (whole-group path) and lmax 6 and 8 (pair-by-pair path; 512-thread
    CTAs at lmax 8)."""
    rng = np.random.default_rng(11)
    L = nat.lib()
    dev = torch.device("cuda", 0)
    for N, lmax in [(7, 4), (6, 5), (5, 6), (4, 8)]:
        pos, _ = random_cluster(rng, N, 40 * nm, 80 * nm, 1200 * nm)
        B = 2 * lmax * (lmax + 2)
        P = N * (N - 1) // 2
        n = P * B * B
        k = 2 * np.pi / (600 * nm)
        dpos = torch.from_numpy(np.concatenate([pos.reshape(-1), pos.reshape(-1)])).to(dev)
        outs = []
        for base in (0, 1):
            # two copies of the cluster: the second at mat_off = n + 2 + base
            sysv = nat.systems_array([(N, lmax, k, 0, base, 0, 0), (N, lmax, k, 3 * N, n + 2 + base, 0, 0)])
            hi = torch.full((2 * n + 4,), float("nan"), dtype=torch.complex64, device=dev)
            lo = torch.full_like(hi, float("nan"))
            nat.check(L.gb_assemble_batch(2, sysv, nat.ptr(dpos), None, nat.ptr(hi), nat.ptr(lo), current_stream(dev)))
            torch.cuda.synchronize()
            outs.append([(t[base: base + n].clone(), t[n + 2 + base: 2 * n + 2 + base].clone()) for t in (hi, lo)])
        for plane in range(2):
            for cl in range(2):
                a, b = outs[0][plane][cl], outs[1][plane][cl]
                assert torch.equal(a.view(torch.int64), b.view(torch.int64)), (N, lmax, plane, cl)
        assert torch.equal(outs[0][0][0].view(torch.int64), outs[0][0][1].view(torch.int64))   # both copies alike


def test_cluster_lmax9_on_the_dense_operator():
    """A cluster of lmax 9 (beyond the packed solvers' lmax 8) through the public API
    solves on the dense operator: p_inc against the oracle's exact solve (1e-10),
    C_ext against the oracle's cross-sections (1e-9)."""
    pos = np.array([[-110, 0, 0], [110, 0, 0], [0, 190, 40]], float) * nm
    mat = gb.constant_material(index=1.6 + 0.05j)
    c = gb.sphere_cluster(position=pos, radius=80 * nm, material=mat, source=gb.plane_wave.from_string("x"),
                          wavelength=500 * nm, lmax=9, method=gb.solver.exact)
    k = float(np.real(c.material_data.k_b))
    T = O.sphere_aggregate_tmatrix(c.position, c.mie_scat.reshape(3, -1), k)
    x = O.solve_linear_system(T, c.p_src.ravel(), "exact").reshape(c.p_inc.shape)
    assert np.max(np.abs(c.p_inc - x)) / np.max(np.abs(x)) < 1e-10
    per = [O.particle_cross_sections(c.p_scat[i], c.p_inc[i], c.p_src[i], k) for i in range(3)]
    cext = sum(np.sum(p[2]) for p in per)
    assert abs(c.cross_sections().extinction - cext) <= 1e-9 * abs(cext)


def test_plugin_lmax9_solves_on_the_dense_operator():
    """The plugin pair sphere_aggregate_tmatrix_jax -> solve_linear_system_jax at lmax 9
    (beyond the packed solvers): the device aggregate is solved as a dense operator,
    p_inc within 1e-10 of the oracle's exact solve."""
    from miepy_gb300 import backend
    rng = np.random.default_rng(21)
    N, lmax = 3, 9
    pos, rad = random_cluster(rng, N, 60 * nm, 90 * nm, 900 * nm)
    # the spheres' own Mie coefficients (n = 1.6 + 0.05i in vacuum at 650 nm): their
    # decay with order keeps (I + T) well conditioned, as for any physical cluster
    md = gb.material_struct([gb.constant_material(index=1.6 + 0.05j)] * N, gb.constant_material(eps=1.0, mu=1.0),
                            wavelength=650 * nm)
    mie, _ = gb.mie_coefficients(rad, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, lmax)
    k = float(np.real(md.k_b))
    rmax = lmax * (lmax + 2)
    p_src = rng.normal(size=(N, 2, rmax)) + 1j * rng.normal(size=(N, 2, rmax))
    agg = backend.sphere_aggregate_tmatrix_jax(pos, mie, k)
    x = backend.solve_linear_system_jax(agg, p_src, gb.solver.exact)
    T = O.sphere_aggregate_tmatrix(pos, mie.reshape(N, -1), k)
    ref = O.solve_linear_system(T, p_src.ravel(), "exact").reshape(N, 2, rmax)
    assert rel(x, ref) < 1e-10


# ------------------------------------------------------------------ solves --
@pytest.mark.parametrize("name", G.EXACT_CASES)
def test_fp64_solve_matches_exact_reference(name):
    g = G.load(name)
    b = batch_from_golden(g).assemble()
    b.solve(tol=1e-14, maxiter=2000)
    assert b.status[0] == 0
    N = g["position"].shape[0]
    x = b.cluster_view(0, b.x)[..., 0].cpu().numpy()
    scale = np.max(np.abs(g["p_inc"]))
    np.testing.assert_allclose(x, g["p_inc"], rtol=1e-10, atol=1e-14 * scale)
    b.epilogue(np.real(g["eps_b"]))
    L = int(g["lmax"])
    ps = b.cluster_view(0, b.p_scat)[..., 0].cpu().numpy()
    pi_ = b.cluster_view(0, b.p_int)[..., 0].cpu().numpy()
    np.testing.assert_allclose(ps, g["p_scat"], rtol=1e-10, atol=1e-14 * np.max(np.abs(g["p_scat"])))
    np.testing.assert_allclose(pi_, g["p_int"], rtol=1e-10, atol=1e-14 * np.max(np.abs(g["p_int"])))
    xs = b.xs[: N * 6 * L].view(N, 3, 2, L).cpu().numpy()
    tot = xs.sum(axis=(0, 2, 3))
    np.testing.assert_allclose(tot, g["cross_sections"], rtol=1e-9)
    ref_per = g["cross_sections_per_multipole"]
    assert rel(xs, ref_per) < 1e-9
    F = b.F[: N * 3].view(N, 3).cpu().numpy()
    T = b.T[: N * 3].view(N, 3).cpu().numpy()
    assert rel(F, g["force"]) < 1e-9
    assert rel(T, g["torque"]) < 1e-9
    b.epilogue(np.real(g["eps_b"]), source=False, want_fields=False)
    assert rel(b.F[: N * 3].view(N, 3).cpu().numpy(), g["force_nosource"]) < 1e-9


@pytest.mark.parametrize("name", ["dimer_lmax6_bicgstab", "ag5_lmax2_bicgstab"])
def test_bicgstab_reference_tolerance_matches_reference_run(name):
    g = G.load(name)
    b = batch_from_golden(g).assemble()
    b.solve(tol=1e-5, maxiter=1000)
    x = b.cluster_view(0, b.x)[..., 0].cpu().numpy()
    np.testing.assert_allclose(x, g["p_inc"], rtol=1e-4, atol=1e-14 * np.max(np.abs(g["p_inc"])))
    # same algorithm, same start: the iterates agree far below the tolerance
    assert rel(x, g["p_inc"]) < 1e-8


@pytest.mark.parametrize("tol,inner", [(1e-8, 1e-4), (1e-10, 1e-4), (1e-5, 1e-4), (1e-8, 1e-6)])
def test_mixed_reported_residual_is_the_true_residual(tol, inner):
    """The mixed solve's residual after its last refinement pass, updated
    incrementally with the complex64 matrix once |r| <= 2.5e4 tol |b|, agrees with
    b - (I + T) x recomputed in double-float, and is below tol."""
    rng = np.random.default_rng(21)
    pos, rad = random_cluster(rng, 60, 50 * nm, 100 * nm, 1400 * nm)
    md = gb.material_struct([gb.constant_material(index=1.5 + 0.01j)] * 60, gb.constant_material(eps=1.0, mu=1.0),
                            wavelength=600 * nm)
    ms, mi = gb.mie_coefficients(rad, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, 4)
    p_src = np.stack([gb.plane_wave.from_string(p).structure(pos, md.k_b, 4) for p in "xy"], axis=-1)
    b = ClusterBatch([dict(position=pos, mie_scat=ms, mie_int=mi, k=float(np.real(md.k_b)), p_src=p_src)], R=2,
                     precision="mixed").assemble()
    b.solve(tol=tol, maxiter=1000, inner_tol=inner, max_refine=8)
    assert np.all(b.status == 0)
    r = (b.b - b.apply(b.x, "mixed")).view(-1, 2).cpu().numpy()
    true = np.linalg.norm(r, axis=0) / np.linalg.norm(b.b.view(-1, 2).cpu().numpy(), axis=0)
    reported = np.asarray(b.resid)
    assert np.all(reported < tol) and np.all(true < tol)
    assert np.all(np.abs(true - reported) <= 0.05 * tol)


def test_mixed_precision_meets_fp64_within_1e6():
    rng = np.random.default_rng(11)
    N, lmax = 40, 4
    pos, rad = random_cluster(rng, N, 50 * nm, 100 * nm, 1200 * nm)
    mat = gb.constant_material(index=1.5 + 0.01j)
    c64 = gb.sphere_cluster(position=pos, radius=rad, material=mat, source=gb.plane_wave.from_string("x"),
                            wavelength=600 * nm, lmax=lmax, precision="mixed", tol=1e-10)
    c64r = gb.sphere_cluster(position=pos, radius=rad, material=mat, source=gb.plane_wave.from_string("x"),
                             wavelength=600 * nm, lmax=lmax, precision="mixed_fp64res", tol=1e-10)
    c128 = gb.sphere_cluster(position=pos, radius=rad, material=mat, source=gb.plane_wave.from_string("x"),
                             wavelength=600 * nm, lmax=lmax, precision="fp64", tol=1e-12)
    e64 = c64.cross_sections().extinction
    e128 = c128.cross_sections().extinction
    assert abs(e64 - e128) / abs(e128) < 1e-6
    assert rel(c64.p_inc, c128.p_inc) < 1e-8
    assert rel(c64r.p_inc, c128.p_inc) < 1e-8
    assert c64.solver_status == 0 and c64r.solver_status == 0
    c32 = gb.sphere_cluster(position=pos, radius=rad, material=mat, source=gb.plane_wave.from_string("x"),
                            wavelength=600 * nm, lmax=lmax, precision="fp32", tol=1e-6)
    assert abs(c32.cross_sections().extinction - e128) / abs(e128) < 1e-4


def test_ragged_batch_equals_individual_solves():
    rng = np.random.default_rng(5)
    specs = []
    k = 2 * np.pi / (600 * nm)
    for N, lmax in ((3, 2), (8, 4), (5, 3), (2, 6)):
        pos, rad = random_cluster(rng, N, 40 * nm, 80 * nm, 900 * nm)
        mie, mint = gb.mie_coefficients(rad, 2.25 + 0.05j, 1.0, 1.0, 1.0, k, lmax)
        p = rng.normal(size=(N, 2, lmax * (lmax + 2), 2)) + 0j
        specs.append(dict(position=pos, mie_scat=mie, mie_int=mint, k=k, p_src=p))
    for prec in ("fp64", "mixed", "mixed_fp64res"):
        bb = ClusterBatch(specs, R=2, precision=prec).assemble()
        bb.solve(tol=1e-12)
        for s, spec in enumerate(specs):
            one = ClusterBatch([spec], R=2, precision=prec).assemble()
            one.solve(tol=1e-12)
            a = bb.cluster_view(s, bb.x).cpu().numpy()
            c = one.cluster_view(0, one.x).cpu().numpy()
            assert rel(a, c) < 1e-10, (prec, s)
            # and against the oracle's exact solution, per right-hand side
            T = O.sphere_aggregate_tmatrix(spec["position"], spec["mie_scat"].reshape(spec["position"].shape[0], -1),
                                           spec["k"])
            for r in range(2):
                ex = O.solve_linear_system(T, spec["p_src"][..., r].ravel(), "exact")
                assert rel(a[..., r].ravel(), ex) < 1e-9


def test_public_cluster_api_dimer():
    g = G.load("dimer_lmax6_exact")
    c = gb.sphere_cluster(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
                          material=gb.constant_material(index=0.2 + 3.0j), source=gb.plane_wave.from_string("x"),
                          wavelength=600 * nm, lmax=6, medium=gb.materials.water(), method=gb.solver.exact)
    np.testing.assert_allclose(c.p_inc, g["p_inc"], rtol=1e-10, atol=1e-14 * np.max(np.abs(g["p_inc"])))
    C = c.cross_sections()
    np.testing.assert_allclose([C.scattering, C.absorption, C.extinction], g["cross_sections"], rtol=1e-9)
    assert rel(c.force(), g["force"]) < 1e-9
    assert rel(c.torque(), g["torque"]) < 1e-9
    for i in range(2):
        Fi = c.force_on_particle(i)
        assert rel(Fi, g["force"][i]) < 1e-9


def test_field_from_particle_matches_reference():
    """E/H_field_from_particle (sphere_cluster.py:150-200) of the dimer at kr >= 9 from
    the particle, with and without the source: 1e-9 of the largest field."""
    g = G.load("dimer_lmax6_field_from_particle")
    c = gb.sphere_cluster(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
                          material=gb.constant_material(index=0.2 + 3.0j), source=gb.plane_wave.from_string("x"),
                          wavelength=600 * nm, lmax=6, medium=gb.materials.water(), method=gb.solver.exact)
    x, y, z = g["field_x"], g["field_y"], g["field_z"]
    assert rel(c.E_field_from_particle(0, x, y, z), g["E0"]) < 1e-9
    assert rel(c.H_field_from_particle(0, x, y, z), g["H0"]) < 1e-9
    assert rel(c.E_field_from_particle(1, x, y, z), g["E1"]) < 1e-9
    assert rel(c.E_field_from_particle(0, x, y, z, source=False), g["E0_nosource"]) < 1e-9


def test_near_fields_match_reference():
    for name in ("dimer_lmax6_exact", "rand12_lmax3_exact"):
        g = G.load(name)
        pos, rad = g["position"], g["radius"]
        lmax = int(g["lmax"])
        N = pos.shape[0]
        dev = torch.device("cuda")
        d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
        x, y, z = g["field_x"], g["field_y"], g["field_z"]
        # keep every device buffer referenced until the kernel has run
        pts = d(np.stack([x, y, z], 1), torch.float64)
        k_int = d(2 * np.pi * g["n"] / g["wavelength"], torch.complex128)
        dpos, drad = d(pos, torch.float64), d(rad, torch.float64)
        dps, dpi = d(g["p_scat"], torch.complex128), d(g["p_int"], torch.complex128)
        out = torch.empty((len(x), 3), dtype=torch.complex128, device=dev)
        nat.check(nat.lib().gb_near_field(N, lmax, nat.ptr(dpos), nat.ptr(drad), nat.ptr(dps), nat.ptr(dpi),
                                          float(g["k_b"]), nat.ptr(k_int), len(x), nat.ptr(pts), 0, 0, 1.0, 0.0, None,
                                          nat.ptr(out), current_stream()))
        torch.cuda.synchronize()
        E = out.cpu().numpy().T
        assert rel(E, g["E_scat_only"]) < 1e-9, name


def test_cluster_fields_match_reference():
    g = G.load("dimer_lmax6_exact")
    c = gb.sphere_cluster(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
                          material=gb.constant_material(index=0.2 + 3.0j), source=gb.plane_wave.from_string("x"),
                          wavelength=600 * nm, lmax=6, medium=gb.materials.water(), method=gb.solver.exact)
    x, y, z = g["field_x"], g["field_y"], g["field_z"]
    inside = np.zeros(x.shape, bool)
    for p_ in c.position:
        inside |= (x - p_[0]) ** 2 + (y - p_[1]) ** 2 + (z - p_[2]) ** 2 < (75 * nm) ** 2
    E, H = c.E_field(x, y, z), c.H_field(x, y, z)
    # outside the spheres: 1e-9 (interior points: test_interior_fields_high_precision)
    assert rel(E[:, ~inside], g["E_total"][:, ~inside]) < 1e-9
    assert rel(H[:, ~inside], g["H_total"][:, ~inside]) < 1e-9


INTERIOR_CASES = {
    "interior_dimer_lmax6": dict(radius=75 * nm, material=gb.constant_material(index=0.2 + 3.0j),
                                 medium=gb.materials.water(), lmax=6),
    "interior_big_lmax8": dict(radius=300 * nm, material=gb.constant_material(index=4.0 + 0.01j), medium=None,
                               lmax=8),
}


@pytest.mark.parametrize("name", list(INTERIOR_CASES))
def test_interior_fields_high_precision(name):
    """Interior fields (j_n of complex k_int r) against the reference's field formula
    evaluated with 40-digit j_n: 1e-9 of the largest field at every point.  Against
    the reference as it is (upward recurrence, cpp/src/special.cpp:20-45): 1e-9 at
    the points where the reference itself is within 1e-10 of the 40-digit value; at
    the others (near the centres, |k_int r| < n) the reference's upward recurrence is
    off by up to 30x the field (interior_dimer_lmax6) and 0.35x (interior_big_lmax8)."""
    g = G.load(name)
    cs = INTERIOR_CASES[name]
    kw = dict(position=g["position"], radius=cs["radius"], material=cs["material"],
              source=gb.plane_wave.from_string("x"), wavelength=600 * nm, lmax=cs["lmax"], method=gb.solver.exact)
    if cs["medium"] is not None:
        kw["medium"] = cs["medium"]
    c = gb.sphere_cluster(**kw)
    x, y, z = g["field_x"], g["field_y"], g["field_z"]
    E, H = c.E_field(x, y, z), c.H_field(x, y, z)
    assert rel(E, g["E_mp"]) < 1e-9
    assert rel(H, g["H_mp"]) < 1e-9
    for F, ref, mp in ((E, g["E_ref"], g["E_mp"]), (H, g["H_ref"], g["H_mp"])):
        scale = np.abs(mp).max()
        ok = np.abs(ref - mp).max(axis=0) <= 1e-10 * scale
        assert ok.sum() >= 20
        assert np.abs(F[:, ok] - ref[:, ok]).max() < 1e-9 * scale


def test_plugin_backend_functions():
    g = G.load("ag5_lmax2_exact")
    from miepy_gb300 import backend
    T = backend.sphere_aggregate_tmatrix_jax(g["position"], g["mie_scat"], g["k_b"])
    assert rel(np.asarray(T), g["agg_tmatrix"]) < 1e-12
    p = backend.solve_linear_system_jax(T, g["p_src"], gb.solver.exact)
    np.testing.assert_allclose(p, g["p_inc"], rtol=1e-10, atol=1e-14 * np.max(np.abs(g["p_inc"])))
    p2 = backend.solve_linear_system_jax(np.asarray(T), g["p_src"], gb.solver.exact)
    np.testing.assert_allclose(p2, g["p_inc"], rtol=1e-10, atol=1e-14 * np.max(np.abs(g["p_inc"])))
    Cs, Ca, Ce = backend.particle_cross_sections_jax(g["p_scat"][0], g["p_inc"][0], g["p_src"][0], g["k_b"])
    ref = g["cross_sections_per_multipole"][0]
    assert rel(np.array([Cs, Ca, Ce]), ref) < 1e-12
    one = backend.sphere_aggregate_tmatrix_jax(g["position"][:1], g["mie_scat"][:1], g["k_b"])
    assert np.all(np.asarray(one) == 0)


def test_plugin_aggregate_edited_like_the_reference():
    """The reference edits the plugin's aggregate: ``agg -= R`` for an interface
    (sphere_cluster.py:704-710) and entry-wise ``agg[i, a, r, j, b, s] += ...`` for
    lattice sums (interactions.py:172-184).  Both give the reference's solutions."""
    from miepy_gb300 import backend
    from oracle import oracle as O
    g = G.load("interface3_lmax3_exact")
    T = backend.sphere_aggregate_tmatrix_jax(g["position"], g["mie_scat"], g["k_b"])
    T -= g["reflection_matrix"]
    p = backend.solve_linear_system_jax(T, g["p_src"], gb.solver.exact)
    assert rel(p, g["p_inc"]) < 1e-10
    g = G.load("periodic_square_dimer_lmax2")
    T = backend.sphere_aggregate_tmatrix_jax(g["position"], g["mie_scat"], g["k_b"])
    lattice = g["agg_tmatrix"] - O.sphere_aggregate_tmatrix(g["position"], g["mie_scat"], g["k_b"]).reshape(T.shape)
    for i in range(2):
        for j in range(2):
            T[i, :, :, j, :, :] += lattice[i, :, :, j, :, :]
    assert rel(np.asarray(T), g["agg_tmatrix"]) < 1e-12
    p = backend.solve_linear_system_jax(T, g["p_src"], gb.solver.exact)
    assert rel(p, g["p_inc"]) < 1e-10


def test_full_size_random_cluster_residual():
    """N = 200, lmax = 4 (D = 9600), two polarisations: the FP64 solution satisfies
    the oracle's own matrix equation (a size-independent check)."""
    rng = np.random.default_rng(2)
    pos, rad = random_cluster(rng, 200, 50 * nm, 100 * nm, 2000 * nm)
    mat = gb.constant_material(index=1.5 + 0.01j)
    c = gb.sphere_cluster(position=pos, radius=rad, material=mat, source=gb.plane_wave.from_string("x"),
                          wavelength=600 * nm, lmax=4, tol=1e-12)
    assert c.solver_status == 0
    T = O.sphere_aggregate_tmatrix(pos, c.mie_scat.reshape(200, -1), c.material_data.k_b)
    r = O.gemv(T, c.p_inc.ravel()) + c.p_inc.ravel() - c.p_src.ravel()
    assert np.linalg.norm(r) / np.linalg.norm(c.p_src) < 1e-11


# ------------------------------------------------- batch reuse and readback --
def _spec(seed, N=12, lmax=3, R=2):
    rng = np.random.default_rng(seed)
    pos, rad = random_cluster(rng, N, 40 * nm, 80 * nm, 900 * nm)
    md = gb.material_struct([gb.constant_material(index=1.6 + 0.05j)] * N, gb.constant_material(eps=1.0, mu=1.0),
                            wavelength=(550 + 20 * seed) * nm)
    ms, mi = gb.mie_coefficients(rad, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, lmax)
    srcs = [gb.plane_wave.from_string("x"), gb.plane_wave.from_string("y")][:R]
    p_src = np.stack([s.structure(pos, md.k_b, lmax) for s in srcs], axis=-1)
    return dict(position=pos, mie_scat=ms, mie_int=mi, k=float(np.real(md.k_b)), p_src=p_src)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_load_reuses_batch_like_a_fresh_one(precision):
    """A batch loaded with a new cluster of the same shape (new positions, Mie
    coefficients, wavenumber and sources) gives exactly what a fresh batch gives;
    to_host returns the same values as the device tensors."""
    a, b = _spec(1), _spec(2)
    reused = ClusterBatch([a], R=2, precision=precision)
    for spec in (a, b):
        reused.load([spec]) if spec is b else None
        reused.assemble().solve(tol=1e-10, inner_tol=1e-4)
        reused.epilogue(1.0)
        out = reused.to_host()
        fresh = ClusterBatch([spec], R=2, precision=precision).assemble()
        fresh.solve(tol=1e-10, inner_tol=1e-4)
        fresh.epilogue(1.0)
        assert np.all(reused.status == 0) and np.all(fresh.status == 0)
        np.testing.assert_array_equal(out["x"], fresh.x.cpu().numpy())
        np.testing.assert_array_equal(out["xs"], fresh.xs.cpu().numpy())
        np.testing.assert_array_equal(out["F"], fresh.F.cpu().numpy())
        np.testing.assert_array_equal(out["T"], fresh.T.cpu().numpy())
    with pytest.raises(ValueError):
        reused.load([_spec(3, N=11)])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotuned_gemv_shapes(precision):
    """gb_autotune_gemv measures the lane shapes of a ragged batch (block sizes 30 and
    70); every shape covers its block, the products with the measured shapes match
    the oracle's matvec (1e-12 FP64, 2e-6 complex64), and a new batch solved with
    them reaches the same solution (1e-8)."""
    specs = [_spec(31, N=9, lmax=3), _spec(32, N=7, lmax=5)]
    b = ClusterBatch(specs, R=2, precision=precision).assemble()
    b.solve(tol=1e-10, inner_tol=1e-4)
    ref = b.x.cpu().numpy()
    shapes = b.autotune()
    assert set(shapes) == {30, 70}
    for B, (lpr, cpl) in shapes.items():
        assert lpr * cpl >= B
    fresh = ClusterBatch(specs, R=2, precision=precision).assemble()
    rng = np.random.default_rng(5)
    x = rng.normal(size=fresh.totals["vec"]) + 1j * rng.normal(size=fresh.totals["vec"])
    y = fresh.apply(torch.from_numpy(x).to(fresh.device), "fp64" if precision == "fp64" else "fp32").cpu().numpy()
    for q, sp in enumerate(specs):
        l = fresh.layout[q]
        T = O.sphere_aggregate_tmatrix(sp["position"], np.asarray(sp["mie_scat"]).reshape(l["N"], -1), sp["k"])
        xs = x[l["vec_off"]: l["vec_off"] + l["D"] * 2].reshape(l["D"], 2)
        want = np.stack([O.gemv(T, xs[:, r]) + xs[:, r] for r in range(2)], axis=1)
        got = y[l["vec_off"]: l["vec_off"] + l["D"] * 2].reshape(l["D"], 2)
        assert rel(got, want) < (1e-12 if precision == "fp64" else 2e-6)
    fresh.solve(tol=1e-10, inner_tol=1e-4)
    assert np.all(fresh.status == 0)
    assert rel(fresh.x.cpu().numpy(), ref) < 1e-8


def test_far_and_spherical_fields_match_reference():
    """E_field / H_field with far=True and/or spherical=True (sphere_cluster.py:244-391,
    expand_E_far / expand_H_far, vsh/expansion.py:45-77,96-108) against the reference's
    own values for the water dimer (fixture dimer_lmax6_far_spherical): 1e-9 of the
    largest component."""
    g = G.load("dimer_lmax6_far_spherical")
    c = gb.sphere_cluster(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
                          material=gb.constant_material(index=0.2 + 3.0j), source=gb.plane_wave.from_string("x"),
                          wavelength=600 * nm, lmax=6, medium=gb.materials.water(), method=gb.solver.exact)
    th, ph = g["theta"], g["phi"]
    cases = [
        (c.E_field(g["x_far"], g["y_far"], g["z_far"], far=True), g["E_far"]),
        (c.H_field(g["x_far"], g["y_far"], g["z_far"], far=True), g["H_far"]),
        (c.E_field(g["r_far"], th, ph, far=True, spherical=True), g["E_far_sph"]),
        (c.H_field(g["r_far"], th, ph, far=True, spherical=True), g["H_far_sph"]),
        (c.E_field(g["r_far"], th, ph, far=True, spherical=True, source=False), g["E_far_scat_sph"]),
        (c.E_field(g["r_near"], th, ph, spherical=True), g["E_near_sph"]),
        (c.H_field(g["r_near"], th, ph, spherical=True), g["H_near_sph"]),
    ]
    for got, want in cases:
        assert rel(got, want) < 1e-9

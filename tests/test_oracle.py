"""CPU tests of the oracle: special functions against scipy/sympy, and the whole
sphere-cluster path against the golden fixtures produced by the reference's own
Python layer."""

import numpy as np
import pytest
import scipy.special as sp

from oracle import oracle as O
from tests import _golden as G


def test_hankel_matches_scipy():
    x = np.linspace(0.2, 30.0, 61)
    for n in range(0, 18):
        ref = sp.spherical_jn(n, x) + 1j * sp.spherical_yn(n, x)
        got = O.spherical_hn(n, x)
        np.testing.assert_allclose(got, ref, rtol=1e-9)
        rec = np.array([O.spherical_hn_recursion(17, xx)[n] for xx in x])
        np.testing.assert_allclose(rec, ref, rtol=1e-9)


def test_real_bessel_matches_scipy():
    x = np.linspace(0.05, 25.0, 73)
    for n in range(0, 15):
        np.testing.assert_allclose(O.riccati_1(n, x) / x, sp.spherical_jn(n, x), rtol=1e-10, atol=1e-300)
        np.testing.assert_allclose(O.spherical_yn(n, x), sp.spherical_yn(n, x), rtol=1e-10)


def test_legendre_no_condon_shortley():
    z = np.linspace(-0.995, 0.995, 37)
    for n in range(0, 18):
        for m in range(-n, n + 1):
            ref = (-1) ** abs(m) * sp.lpmv(abs(m), n, z)
            if m < 0:
                ref = ref * (-1) ** m * sp.factorial(n + m) / sp.factorial(n - m)
            got = O.associated_legendre(np.full(z.shape, n), m, z)
            np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())


def test_legendre_recursion_packing():
    z = 0.37
    tab = O.associated_legendre_recursion(9, z)
    for n in range(0, 10):
        for m in range(-n, n + 1):
            assert tab[n * (n + 2) - n + m] == pytest.approx(O.associated_legendre(n, m, z), rel=1e-13, abs=1e-300)


def test_pi_tau_against_definitions():
    th = np.linspace(0.05, np.pi - 0.05, 19)
    h = 1e-6
    for n in range(1, 9):
        for m in range(-n, n + 1):
            P = O.associated_legendre(np.full(th.shape, n), m, np.cos(th))
            np.testing.assert_allclose(O.pi_func(n, m, th), m / np.sin(th) * P, rtol=1e-12, atol=1e-14)
            dP = (O.associated_legendre(np.full(th.shape, n), m, np.cos(th + h)) -
                  O.associated_legendre(np.full(th.shape, n), m, np.cos(th - h))) / (2 * h)
            np.testing.assert_allclose(O.tau_func(n, m, th), dP, rtol=1e-6, atol=1e-6 * np.abs(dP).max() + 1e-12)


def test_wigner3j_and_gaunt_against_sympy():
    wig = pytest.importorskip("sympy.physics.wigner")
    rng = np.random.default_rng(1)
    for _ in range(300):
        j1, j2 = rng.integers(0, 9, size=2)
        j3 = rng.integers(abs(j1 - j2), j1 + j2 + 1)
        m1 = rng.integers(-j1, j1 + 1)
        m2 = rng.integers(-j2, j2 + 1)
        m3 = -m1 - m2
        if abs(m3) > j3:
            continue
        ref = float(wig.wigner_3j(int(j1), int(j2), int(j3), int(m1), int(m2), int(m3)))
        assert O.wigner_3j(j1, j2, j3, m1, m2, m3) == pytest.approx(ref, rel=1e-12, abs=1e-15)
    # recursive Gaunt batch against the direct 3j products (the reference's own self-check)
    for n in range(1, 7):
        for v in range(1, n + 1):
            for m in range(-n, n + 1):
                for u in range(-v, v + 1):
                    a, b = O.gaunt_batch(m, n, u, v)
                    for q in range(len(a)):
                        p = n + v - 2 * q
                        assert a[q] == pytest.approx(O.a_func(m, n, u, v, p), rel=1e-9, abs=1e-12)
                    for q in range(1, len(b)):
                        p = n + v - 2 * q
                        assert b[q] == pytest.approx(O.b_func(m, n, u, v, p), rel=1e-9, abs=1e-12)


def test_translation_symmetries():
    """Parity/swap symmetries of A and B that the assembler relies on."""
    r, th, ph, k = 1.0, 0.7, 0.3, 0.8
    for n in range(1, 4):
        for m in range(-n, n + 1):
            for v in range(1, 4):
                for u in range(-v, v + 1):
                    A, B = O.vsh_translation(m, n, u, v, r, th, ph, k, O.MODE_OUTGOING)
                    A2, B2 = O.vsh_translation(m, n, u, v, r, np.pi - th, np.pi + ph, k, O.MODE_OUTGOING)
                    assert A2 == pytest.approx((-1) ** (n + v) * A, rel=1e-10, abs=1e-14)
                    assert B2 == pytest.approx((-1) ** (n + v + 1) * B, rel=1e-10, abs=1e-14)
                    A3, B3 = O.vsh_translation(-u, v, -m, n, r, th, ph, k, O.MODE_OUTGOING)
                    assert A3 == pytest.approx((-1) ** (m + u) * A, rel=1e-10, abs=1e-14)
                    assert B3 == pytest.approx((-1) ** (m + u + 1) * B, rel=1e-10, abs=1e-14)


@pytest.mark.parametrize("name", ["dimer_lmax6_exact", "ag5_lmax2_exact"])
def test_oracle_aggregate_matches_golden(name):
    g = G.load(name)
    N = g["position"].shape[0]
    T = O.sphere_aggregate_tmatrix(g["position"], g["mie_scat"].reshape(N, -1), g["k_b"])
    ref = g["agg_tmatrix"].reshape(T.shape)
    assert np.max(np.abs(T - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("name", G.EXACT_CASES)
def test_oracle_solve_and_observables_match_golden(name):
    g = G.load(name)
    N, lmax = g["position"].shape[0], int(g["lmax"])
    rmax = lmax * (lmax + 2)
    T = O.sphere_aggregate_tmatrix(g["position"], g["mie_scat"].reshape(N, -1), g["k_b"])
    x = O.solve_linear_system(T, g["p_src"].ravel(), "exact").reshape(N, 2, rmax)
    scale = np.max(np.abs(g["p_inc"]))
    np.testing.assert_allclose(x, g["p_inc"], rtol=1e-10, atol=1e-14 * scale)
    per = np.array([[v for v in O.particle_cross_sections(g["p_scat"][i], g["p_inc"][i], g["p_src"][i], g["k_b"])]
                    for i in range(N)]).reshape(N, 3, 2, lmax)
    np.testing.assert_allclose(per, g["cross_sections_per_multipole"], rtol=1e-12, atol=1e-30)
    F = O.force_all(g["p_scat"], g["p_inc"], g["k_b"], np.real(g["eps_b"]))
    np.testing.assert_allclose(F, g["force"], rtol=1e-12, atol=1e-40)


@pytest.mark.parametrize("name", ["dimer_lmax6_bicgstab", "ag5_lmax2_bicgstab"])
def test_oracle_bicgstab_matches_golden(name):
    """Eigen-style BiCGSTAB (tol 1e-5) reproduces the reference pipeline's iterate."""
    g = G.load(name)
    N, lmax = g["position"].shape[0], int(g["lmax"])
    T = O.sphere_aggregate_tmatrix(g["position"], g["mie_scat"].reshape(N, -1), g["k_b"])
    x = O.solve_linear_system(T, g["p_src"].ravel(), "bicgstab").reshape(g["p_inc"].shape)
    scale = np.max(np.abs(g["p_inc"]))
    np.testing.assert_allclose(x, g["p_inc"], rtol=1e-9, atol=1e-13 * scale)

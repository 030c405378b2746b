"""Single-sphere Mie coefficients, vectorised over particles and orders.

Same formulas and the same scipy Bessel routines as the reference's
mie_sphere_scattering_coefficients / mie_sphere_interior_coefficients
(mie_single/mie_sphere.py:16-76 with special_functions.py:127-153), evaluated for
all (particle, n) at once instead of one Python call per pair.
"""

from __future__ import annotations

import numpy as np
from scipy import special as sp


def _riccati_1(n, x):
    jn = sp.spherical_jn(n, x)
    jnp = sp.spherical_jn(n, x, derivative=True)
    return x * jn, jn + x * jnp


def _riccati_2(n, x):
    yn = sp.spherical_yn(n, x)
    ynp = sp.spherical_yn(n, x, derivative=True)
    return x * yn, yn + x * ynp


def mie_coefficients(radius, eps, mu, eps_b, mu_b, k, lmax, conducting=None):
    """Returns (mie_scat, mie_int), each [N, 2, lmax] complex: (a_n, b_n) and (c_n, d_n)."""
    radius = np.asarray(radius, dtype=float).reshape(-1)
    N = radius.shape[0]
    eps = np.broadcast_to(np.asarray(eps, dtype=complex), (N,))
    mu = np.broadcast_to(np.asarray(mu, dtype=complex), (N,))
    cond = np.zeros(N, bool) if conducting is None else np.broadcast_to(np.asarray(conducting, bool), (N,))
    n = np.arange(1, lmax + 1)[None, :]
    x = (k * radius)[:, None] * np.ones((1, lmax))
    m = (eps / eps_b) ** 0.5
    mt = m * mu_b / mu
    m, mt = m[:, None], mt[:, None]
    j0, j1 = _riccati_1(n, x)
    y0, y1 = _riccati_2(n, x)
    h0, h1 = j0 + 1j * y0, j1 + 1j * y1
    jm0, jm1 = _riccati_1(n, m * x)
    with np.errstate(all="ignore"):
        a = (mt * jm0 * j1 - j0 * jm1) / (mt * jm0 * h1 - h0 * jm1)
        b = (jm0 * j1 - mt * j0 * jm1) / (jm0 * h1 - mt * h0 * jm1)
        c = (m * j0 * h1 - m * h0 * j1) / (jm0 * h1 - mt * h0 * jm1)
        d = (m * j0 * h1 - m * h0 * j1) / (mt * jm0 * h1 - h0 * jm1)
    if np.any(cond):
        a = np.where(cond[:, None], j1 / h1, a)
        b = np.where(cond[:, None], j0 / h0, b)
        c = np.where(cond[:, None], 0.0, c)
        d = np.where(cond[:, None], 0.0, d)
    mie_scat = np.stack([a, b], axis=1).astype(complex)
    mie_int = np.stack([c, d], axis=1).astype(complex)
    return mie_scat, mie_int

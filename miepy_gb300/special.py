"""Host-side angular functions for source decompositions (numpy, vectorised).

Conventions of the reference's C++ module: associated Legendre functions without
the Condon-Shortley phase (GSL_SF_LEGENDRE_NONE, cpp/src/special.cpp:148-204),
pi_func / tau_func with their exact limits at theta = 0 and pi
(cpp/src/special.cpp:209-270), E_mn (cpp/src/vsh_functions.cpp:56-58).
"""

from __future__ import annotations

from math import factorial

import numpy as np


def _legendre_table(nmax, x):
    """P[n][m] for 0 <= m <= n <= nmax (m >= 0, no Condon-Shortley phase)."""
    x = np.asarray(x, dtype=float)
    u = np.sqrt(np.maximum(0.0, (1.0 - x) * (1.0 + x)))
    P = np.zeros((nmax + 1, nmax + 1) + x.shape)
    P[0, 0] = 1.0
    for m in range(1, nmax + 1):
        P[m, m] = (2 * m - 1) * u * P[m - 1, m - 1]
    for m in range(0, nmax):
        P[m + 1, m] = x * (2 * m + 1) * P[m, m]
    for m in range(0, nmax + 1):
        for n in range(m + 2, nmax + 1):
            P[n, m] = ((2 * n - 1) * x * P[n - 1, m] - (n + m - 1) * P[n - 2, m]) / (n - m)
    return P


def _neg_factor(n, m):
    am = abs(m)
    return (-1) ** am * factorial(n - am) / factorial(n + am)


def associated_legendre(n, m, x):
    if abs(m) > n:
        return np.zeros_like(np.asarray(x, dtype=float))
    P = _legendre_table(n, x)[n, abs(m)]
    return P * _neg_factor(n, m) if m < 0 else P


def pi_func(n, m, theta):
    theta = np.asarray(theta, dtype=float)
    out = np.empty_like(theta)
    at0, atpi = theta == 0, theta == np.pi
    gen = ~(at0 | atpi)
    if np.any(gen):
        t = theta[gen]
        out[gen] = m / np.sin(t) * associated_legendre(n, m, np.cos(t))
    lim0 = n * (n + 1) / 2.0 if m == 1 else (0.5 if m == -1 else 0.0)
    limpi = (-1) ** (n + 1) * (n * (n + 1) / 2.0 if m == 1 else (0.5 if m == -1 else 0.0))
    out[at0] = lim0
    out[atpi] = limpi
    return out if out.shape else float(out)


def tau_func(n, m, theta):
    theta = np.asarray(theta, dtype=float)
    out = np.empty_like(theta)
    at0, atpi = theta == 0, theta == np.pi
    gen = ~(at0 | atpi)
    if np.any(gen):
        t = theta[gen]
        am = abs(m)
        P = _legendre_table(n + 1, np.cos(t))
        pp1 = P[n, am + 1] if am + 1 <= n else 0.0
        pm1 = P[n, am - 1] if am >= 1 else -P[n, 1] / (n * (n + 1))
        d = 0.5 * ((n + am) * (n - am + 1) * pm1 - pp1)
        out[gen] = d * _neg_factor(n, m) if m < 0 else d
    lim0 = n * (n + 1) / 2.0 if m == 1 else (-0.5 if m == -1 else 0.0)
    limpi = (-1) ** n * (n * (n + 1) / 2.0 if m == 1 else (-0.5 if m == -1 else 0.0))
    out[at0] = lim0
    out[atpi] = limpi
    return out if out.shape else float(out)


def Emn(m, n):
    return (1j) ** n * np.sqrt((2 * n + 1) * factorial(n - m) / (n * (n + 1) * factorial(n + m)))

"""Rotation of VSH expansion coefficients (Wigner-D matrices).

Replaces vsh_rotation_matrix / rotate_expansion_coefficients
(src/miepy/vsh/vsh_rotation.py:8-52), which take their D-matrices from the
``spherical`` package.  Here they come from the closed-form Wigner small-d sum.

Convention.  For a rotation R = Rz(alpha) Ry(beta) Rz(gamma) (active, ZYZ Euler
angles) the standard D-matrix is
    D^n_{m'm} = exp(-i m' alpha) d^n_{m'm}(beta) exp(-i m gamma),
    d^n_{m'm}(beta) = sum_s (-1)^(m'-m+s) sqrt((n+m')!(n-m')!(n+m)!(n-m)!)
                      / ((n+m-s)! s! (m'-m+s)! (n-m'-s)!)
                      cos(beta/2)^(2n+m-m'-2s) sin(beta/2)^(m'-m+2s),
and it rotates spherical harmonics as Y_n^m(R^-1 r) = sum_m' D^n_{m'm} Y_n^m'(r).
The package's VSH (and the reference's) are built from E_mn P_n^m(cos theta)
e^{i m phi} without the Condon-Shortley phase; that scalar is
i^n sqrt(4 pi / (n (n+1))) (-1)^m Y_n^m, so the coefficients of the rotated field
R E(R^-1 r) are
    p'_{m'} = sum_m (-1)^(m - m') D^n_{m'm} p_m,
separately for every order n and for the electric and magnetic halves.  The
orientation of a beam with angles (theta, phi) is Rz(phi) Ry(theta)
(quaternion.from_spherical_coords), i.e. alpha = phi, beta = theta, gamma = 0.
"""

from __future__ import annotations

from math import factorial

import numpy as np

from .modes import lmax_to_rmax


def wigner_small_d(n: int, beta: float) -> np.ndarray:
    """d^n_{m'm}(beta) as a [2n+1, 2n+1] array, rows m' = -n..n, columns m = -n..n."""
    c, s = np.cos(beta / 2), np.sin(beta / 2)
    out = np.zeros((2 * n + 1, 2 * n + 1))
    for mp in range(-n, n + 1):
        for m in range(-n, n + 1):
            pre = np.sqrt(float(factorial(n + mp) * factorial(n - mp) * factorial(n + m) * factorial(n - m)))
            tot = 0.0
            for k in range(max(0, m - mp), min(n + m, n - mp) + 1):
                den = factorial(n + m - k) * factorial(k) * factorial(mp - m + k) * factorial(n - mp - k)
                tot += (-1) ** (mp - m + k) / den * c ** (2 * n + m - mp - 2 * k) * s ** (mp - m + 2 * k)
            out[mp + n, m + n] = pre * tot
    return out


def vsh_rotation_matrix(n: int, alpha: float, beta: float, gamma: float = 0.0) -> np.ndarray:
    """[2n+1, 2n+1] matrix M with p' = M p for the order-n coefficients of a field
    rotated by Rz(alpha) Ry(beta) Rz(gamma)."""
    m = np.arange(-n, n + 1)
    D = np.exp(-1j * m[:, None] * alpha) * wigner_small_d(n, beta) * np.exp(-1j * m[None, :] * gamma)
    return D * (-1.0) ** np.subtract.outer(m, m)


def rotate_expansion_coefficients(p_exp, alpha: float, beta: float, gamma: float = 0.0) -> np.ndarray:
    """p_exp [..., 2, rmax] -> the coefficients of the rotated field, same shape."""
    p_exp = np.asarray(p_exp, dtype=complex)
    rmax = p_exp.shape[-1]
    lmax = int(round(np.sqrt(1 + rmax) - 1))
    out = np.empty_like(p_exp)
    for n in range(1, lmax + 1):
        M = vsh_rotation_matrix(n, alpha, beta, gamma)
        hi = lmax_to_rmax(n)
        sl = np.s_[hi - (2 * n + 1): hi]
        out[..., sl] = np.einsum("ab,...b->...a", M, p_exp[..., sl])
    return out


def rotation_matrix(alpha: float, beta: float, gamma: float = 0.0) -> np.ndarray:
    """The 3 x 3 matrix Rz(alpha) Ry(beta) Rz(gamma)."""
    def rz(a):
        return np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1.0]])

    ry = np.array([[np.cos(beta), 0, np.sin(beta)], [0, 1.0, 0], [-np.sin(beta), 0, np.cos(beta)]])
    return rz(alpha) @ ry @ rz(gamma)

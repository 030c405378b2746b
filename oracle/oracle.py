"""CPU oracle -- TEST INFRASTRUCTURE ONLY.

numpy-level access to ``oracle/src/oracle_miepy.cpp``, the C++17 restatement of
the native module of johnaparker/miepy (``cpp/src/*.cpp``).  It is loaded only by
the parity tests, by ``__graft_entry__.smoke()`` (as the checker) and by the
CPU-baseline leg of ``bench.py``.  The product package ``miepy_gb300`` never
imports it.

Array conventions follow the reference's pybind11 layer: complex128 arrays,
row-major, ``mie`` as ``[N, 2*lmax]``, aggregate matrices as ``[D, D]``.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "build", "liboracle_miepy.so")

_lib = None
_lock = threading.Lock()

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)

# vsh_mode enum order of cpp/src/vsh_functions.hpp:10-15
MODE_OUTGOING, MODE_INGOING, MODE_INCIDENT, MODE_INTERIOR = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile the oracle library with make (g++ -O3 -fopenmp)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            _declare(L)
            _lib = L
    return _lib


def _declare(L):
    c_int, c_double = ctypes.c_int, ctypes.c_double
    sig = {
        "orc_num_threads": (c_int, []),
        "orc_set_num_threads": (None, [c_int]),
        "orc_factorial": (c_double, [c_double]),
        "orc_spherical_jn": (None, [c_int, _I, _D, c_int, _D]),
        "orc_spherical_yn": (None, [c_int, _I, _D, c_int, _D]),
        "orc_spherical_hn": (None, [c_int, _I, _D, c_int, c_int, _D]),
        "orc_spherical_hn_recursion": (None, [c_int, c_double, _D]),
        "orc_riccati": (None, [c_int, c_int, _I, _D, c_int, _D]),
        "orc_associated_legendre": (None, [c_int, _I, _I, _D, _D]),
        "orc_associated_legendre_recursion": (None, [c_int, c_double, _D]),
        "orc_pi_func": (None, [c_int, _I, _I, _D, _D]),
        "orc_tau_func": (None, [c_int, _I, _I, _D, _D]),
        "orc_wigner_3j": (c_double, [c_int] * 6),
        "orc_a_func": (c_double, [c_int] * 5),
        "orc_b_func": (c_double, [c_int] * 5),
        "orc_wigner_3j_batch": (c_int, [c_int] * 5 + [_I, _D, c_int]),
        "orc_gaunt_batch": (None, [c_int] * 4 + [_D, _I, _D, _I]),
        "orc_vsh_translation": (None, [c_int, c_int, c_int, c_int, c_int, _D, _D, _D, c_double, c_int, _D]),
        "orc_vsh_cache_entry": (None, [c_int] * 4 + [_D, _I, _I, _D, _D]),
        "orc_sphere_aggregate_tmatrix": (None, [c_int, c_int, _D, _D, c_double, _D]),
        "orc_particle_aggregate_tmatrix": (None, [c_int, c_int, _D, _D, c_double, _D]),
        "orc_reflection_matrix_nia": (None, [c_int, c_int, _D, _D, c_double, c_double, c_double, c_double, _D]),
        "orc_sphere_aggregate_tmatrix_periodic": (None, [c_int, c_int, _D, _D, c_double, c_int, _D, _D, _D]),
        "orc_solve_linear_system": (c_int, [c_int, _D, _D, c_int, c_double, c_int, _D, _D]),
        "orc_bicgstab_plain": (c_int, [c_int, _D, _D, c_int, c_double, _D, _D]),
        "orc_solve_linear_system_precond": (c_int, [c_int, _D, _D, c_int, _D, c_int, c_double, c_int, _D, _D]),
        "orc_bicgstab_precond": (c_int, [c_int, _D, _D, _D, c_int, c_int, c_double, _D, _D]),
        "orc_gemv": (None, [c_int, _D, _D, _D]),
        "orc_particle_cross_sections": (None, [c_int, _D, _D, _D, c_double, _D]),
        "orc_cluster_cross_sections": (None, [c_int, _D, _D, c_double, _D]),
        "orc_force": (None, [c_int, _D, _D, c_double, c_double, _D]),
        "orc_torque": (None, [c_int, _D, _D, c_double, c_double, _D]),
        "orc_force_all": (None, [c_int, c_int, _D, _D, c_double, c_double, _D]),
        "orc_torque_all": (None, [c_int, c_int, _D, _D, c_double, c_double, _D]),
        "orc_Emn": (None, [c_int, c_int, _D]),
        "orc_vsh_electric": (None, [c_int, c_int, c_int, c_double, c_double, c_double, c_double, _D]),
        "orc_vsh_magnetic": (None, [c_int, c_int, c_int, c_double, c_double, c_double, c_double, _D]),
        "orc_expand_E_cluster": (None, [c_int, c_int, _D, _D, c_int, c_int, _D, _D, _D, c_double, _D]),
        "orc_integrate_phase": (None, [_D, _D, c_double, c_int, c_int, _D, c_int, _D, _D, _D]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def mode_value(mode) -> int:
    """Accept an int, an enum member with .value, or a name."""
    if isinstance(mode, (int, np.integer)):
        return int(mode)
    if hasattr(mode, "value"):
        return int(mode.value)
    return {"outgoing": 0, "ingoing": 1, "incident": 2, "interior": 3}[str(mode)]


# ------------------------------------------------------------------ threads --
def num_threads() -> int:
    return lib().orc_num_threads()


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


# --------------------------------------------------------- special functions --
def _bcast(*arrs):
    b = np.broadcast_arrays(*[np.asarray(a) for a in arrs])
    return b, b[0].shape


def spherical_jn(n, z, derivative=False):
    (n, z), shape = _bcast(n, z)
    nn = _i32(n.ravel())
    zz = _c128(z.ravel()).view(np.float64)
    out = np.empty(nn.size, dtype=np.complex128)
    lib().orc_spherical_jn(nn.size, _ip(nn), _dp(zz), int(bool(derivative)), _dp(out.view(np.float64)))
    return out.reshape(shape) if shape else out[0]


def spherical_yn(n, z, derivative=False):
    (n, z), shape = _bcast(n, z)
    nn = _i32(n.ravel())
    zz = _f64(z.ravel())
    out = np.empty(nn.size, dtype=np.float64)
    lib().orc_spherical_yn(nn.size, _ip(nn), _dp(zz), int(bool(derivative)), _dp(out))
    return out.reshape(shape) if shape else out[0]


def _hn(n, z, derivative, second):
    (n, z), shape = _bcast(n, z)
    nn = _i32(n.ravel())
    zz = _f64(np.real(z).ravel())
    out = np.empty(nn.size, dtype=np.complex128)
    lib().orc_spherical_hn(nn.size, _ip(nn), _dp(zz), int(bool(derivative)), int(second), _dp(out.view(np.float64)))
    return out.reshape(shape) if shape else out[0]


def spherical_hn(n, z, derivative=False):
    return _hn(n, z, derivative, 0)


def spherical_hn_2(n, z, derivative=False):
    return _hn(n, z, derivative, 1)


def spherical_hn_recursion(nmax, z):
    out = np.empty(nmax + 1, dtype=np.complex128)
    lib().orc_spherical_hn_recursion(int(nmax), float(z), _dp(out.view(np.float64)))
    return out


def _riccati(kind, n, z, derivative):
    (n, z), shape = _bcast(n, z)
    nn = _i32(n.ravel())
    zz = _f64(z.ravel())
    out = np.empty(nn.size, dtype=np.float64)
    lib().orc_riccati(kind, nn.size, _ip(nn), _dp(zz), int(bool(derivative)), _dp(out))
    return out.reshape(shape) if shape else out[0]


def riccati_1(n, z, derivative=False):
    return _riccati(1, n, z, derivative)


def riccati_2(n, z, derivative=False):
    return _riccati(2, n, z, derivative)


def riccati_3(n, z, derivative=False):
    return _riccati(3, n, z, derivative)


def associated_legendre(n, m, z, derivative=False):
    (n, m, z), shape = _bcast(n, m, z)
    nn, mm, zz = _i32(n.ravel()), _i32(m.ravel()), _f64(z.ravel())
    out = np.empty(nn.size, dtype=np.float64)
    if derivative:   # the reference returns 0 for the unimplemented derivative
        out[:] = 0.0
    else:
        lib().orc_associated_legendre(nn.size, _ip(nn), _ip(mm), _dp(zz), _dp(out))
    return out.reshape(shape) if shape else out[0]


def associated_legendre_recursion(nmax, z):
    out = np.empty(nmax * (nmax + 2) + 1, dtype=np.float64)
    lib().orc_associated_legendre_recursion(int(nmax), float(z), _dp(out))
    return out


def _pitau(fn, n, m, theta):
    (n, m, t), shape = _bcast(n, m, theta)
    nn, mm, tt = _i32(n.ravel()), _i32(m.ravel()), _f64(t.ravel())
    out = np.empty(nn.size, dtype=np.float64)
    fn(nn.size, _ip(nn), _ip(mm), _dp(tt), _dp(out))
    return out.reshape(shape) if shape else out[0]


def pi_func(n, m, theta):
    return _pitau(lib().orc_pi_func, n, m, theta)


def tau_func(n, m, theta):
    return _pitau(lib().orc_tau_func, n, m, theta)


def wigner_3j(j1, j2, j3, m1, m2, m3):
    return lib().orc_wigner_3j(int(j1), int(j2), int(j3), int(m1), int(m2), int(m3))


def a_func(m, n, u, v, p):
    return lib().orc_a_func(int(m), int(n), int(u), int(v), int(p))


def b_func(m, n, u, v, p):
    return lib().orc_b_func(int(m), int(n), int(u), int(v), int(p))


def wigner_3j_batch(j2, j3, m1, m2, m3):
    cap = 2 * (j2 + j3) + 4
    out = np.empty(cap, dtype=np.float64)
    jmin = ctypes.c_int(0)
    c = lib().orc_wigner_3j_batch(int(j2), int(j3), int(m1), int(m2), int(m3), ctypes.byref(jmin), _dp(out), cap)
    return jmin.value, jmin.value + c - 1, out[:max(c, 0)].copy()


def gaunt_batch(m, n, u, v):
    a = np.empty(n + v + 2, dtype=np.float64)
    b = np.empty(n + v + 2, dtype=np.float64)
    na, nb = ctypes.c_int(0), ctypes.c_int(0)
    lib().orc_gaunt_batch(int(m), int(n), int(u), int(v), _dp(a), ctypes.byref(na), _dp(b), ctypes.byref(nb))
    return a[:na.value].copy(), b[:nb.value].copy()


def vsh_cache_entry(n, m, v, u):
    f = np.empty(2, dtype=np.float64)
    A = np.zeros(2 * (n + 2), dtype=np.float64)
    B = np.zeros(2 * (n + 2), dtype=np.float64)
    qa, qb = ctypes.c_int(0), ctypes.c_int(0)
    lib().orc_vsh_cache_entry(int(n), int(m), int(v), int(u), _dp(f), ctypes.byref(qa), ctypes.byref(qb), _dp(A), _dp(B))
    Ac = A.view(np.complex128)[: qa.value + 1].copy()
    Bc = B.view(np.complex128)[: qb.value + 1].copy()
    return complex(f[0], f[1]), qa.value, qb.value, Ac, Bc


# ------------------------------------------------------------- translations --
def vsh_translation_numpy(m, n, u, v, rad, theta, phi, k, mode):
    rad, theta, phi = (_f64(np.atleast_1d(a)) for a in (rad, theta, phi))
    out = np.empty((rad.size, 2), dtype=np.complex128)
    lib().orc_vsh_translation(rad.size, int(m), int(n), int(u), int(v), _dp(rad), _dp(theta), _dp(phi), float(k),
                              mode_value(mode), _dp(out.view(np.float64)))
    return np.ascontiguousarray(out.T)


def vsh_translation(m, n, u, v, rad, theta, phi, k, mode):
    r = vsh_translation_numpy(m, n, u, v, [rad], [theta], [phi], k, mode)
    return complex(r[0, 0]), complex(r[1, 0])


def sphere_aggregate_tmatrix(positions, mie, k):
    """positions [N,3], mie [N, 2*lmax] (or [N,2,lmax]) -> T_agg [D, D] c128."""
    pos = _f64(positions).reshape(-1, 3)
    N = pos.shape[0]
    mie = _c128(mie).reshape(N, -1)
    lmax = mie.shape[1] // 2
    rmax = lmax * (lmax + 2)
    D = 2 * rmax * N
    out = np.empty((D, D), dtype=np.complex128)
    lib().orc_sphere_aggregate_tmatrix(N, lmax, _dp(pos), _dp(mie.view(np.float64)), float(np.real(k)),
                                       _dp(out.view(np.float64)))
    return out


def particle_aggregate_tmatrix(positions, tmatrix, k):
    """positions [N,3], tmatrix [N, 2*rmax, 2*rmax] (or [N,2,rmax,2,rmax]) -> T_agg [D, D]
    c128 (cpp/src/interactions.cpp:416-462)."""
    pos = _f64(positions).reshape(-1, 3)
    N = pos.shape[0]
    T = _c128(tmatrix).reshape(N, -1)
    B = int(round(np.sqrt(T.shape[1])))
    rmax = B // 2
    D = B * N
    out = np.empty((D, D), dtype=np.complex128)
    lib().orc_particle_aggregate_tmatrix(N, rmax, _dp(pos), _dp(np.ascontiguousarray(T).view(np.float64)),
                                         float(np.real(k)), _dp(out.view(np.float64)))
    return out


def reflection_matrix_nia(positions, mie, k, reflection, z):
    """Reflection matrix of a planar interface at height z (cpp/src/interactions.cpp:464-512):
    positions [N,3], mie [N, 2*lmax] (or [N,2,lmax]), reflection coefficient r0 ->
    R [D, D] c128, subtracted from the aggregate T-matrix by the reference."""
    pos = _f64(positions).reshape(-1, 3)
    N = pos.shape[0]
    mie = _c128(mie).reshape(N, -1)
    lmax = mie.shape[1] // 2
    D = 2 * lmax * (lmax + 2) * N
    out = np.empty((D, D), dtype=np.complex128)
    r = complex(reflection)
    lib().orc_reflection_matrix_nia(N, lmax, _dp(pos), _dp(mie.view(np.float64)), float(np.real(k)), r.real, r.imag,
                                    float(z), _dp(out.view(np.float64)))
    return out


def sphere_aggregate_tmatrix_periodic(positions, mie, k, cells, k_hat):
    """Aggregate T-matrix of a periodic cluster (src/miepy/interactions.py:153-186):
    positions [N,3], mie [N,2,lmax], the lattice cells [ncell,3] (the symmetry's
    generate(5000) in the reference), the source's unit wave vector k_hat -> [D, D] c128."""
    pos = _f64(positions).reshape(-1, 3)
    N = pos.shape[0]
    mie = _c128(mie).reshape(N, -1)
    lmax = mie.shape[1] // 2
    D = 2 * lmax * (lmax + 2) * N
    cells = _f64(cells).reshape(-1, 3)
    out = np.empty((D, D), dtype=np.complex128)
    lib().orc_sphere_aggregate_tmatrix_periodic(N, lmax, _dp(pos), _dp(mie.view(np.float64)), float(np.real(k)),
                                                cells.shape[0], _dp(cells), _dp(_f64(k_hat).reshape(3)),
                                                _dp(out.view(np.float64)))
    return out


def solve_linear_system_profiled(T, b, method="bicgstab", tol=1e-5, maxiter=1000):
    """(I + T) x = b.  Returns (x, iterations, relative residual)."""
    T = _c128(T)
    D = T.shape[0]
    T = T.reshape(D, D)
    b = _c128(b).reshape(D)
    x = np.empty(D, dtype=np.complex128)
    err = ctypes.c_double(0.0)
    meth = 1 if (getattr(method, "name", method) == "exact" or method == 1) else 0
    it = lib().orc_solve_linear_system(D, _dp(T.view(np.float64)), _dp(b.view(np.float64)), meth, float(tol),
                                       int(maxiter), _dp(x.view(np.float64)), ctypes.byref(err))
    if it < 0:
        raise np.linalg.LinAlgError("singular interaction matrix")
    return x, it, err.value


def solve_linear_system(T, b, method="bicgstab", tol=1e-5, maxiter=1000):
    return solve_linear_system_profiled(T, b, method, tol, maxiter)[0]


def bicgstab(A, b, maxiter=1000, tolerance=1e-5):
    """Hand-written BiCGSTAB of the reference (x0 = b). Returns (x, iters, residual)."""
    A = _c128(A)
    D = A.shape[0]
    b = _c128(b).reshape(D)
    x = np.empty(D, dtype=np.complex128)
    err = ctypes.c_double(0.0)
    it = lib().orc_bicgstab_plain(D, _dp(A.view(np.float64)), _dp(b.view(np.float64)), int(maxiter),
                                  float(tolerance), _dp(x.view(np.float64)), ctypes.byref(err))
    return x, it, err.value


def build_block_preconditioner_sphere(mie_scat, lmax):
    """(M_inv_blocks [N*bs, bs], bs) with the diagonal 1 / (1 + a_n), 1 where
    |1 + a_n| < 1e-12 (src/miepy/interactions.py:9-39)."""
    mie = np.asarray(mie_scat, dtype=complex).reshape(-1, 2, lmax)
    N = mie.shape[0]
    rmax = lmax * (lmax + 2)
    bs = 2 * rmax
    M = np.zeros((N * bs, bs), dtype=complex)
    ns = np.concatenate([np.full(2 * n + 1, n) for n in range(1, lmax + 1)])
    for i in range(N):
        for a in range(2):
            for r in range(rmax):
                val = 1.0 + mie[i, a, ns[r] - 1]
                M[i * bs + a * rmax + r, a * rmax + r] = 1.0 if abs(val) < 1e-12 else 1.0 / val
    return M, bs


def build_block_preconditioner_particle(tmatrix):
    """(M_inv_blocks, bs) with blocks inv(I + T_i), identity where singular
    (src/miepy/interactions.py:42-68)."""
    tm = np.asarray(tmatrix, dtype=complex)
    N, bs = tm.shape[0], 2 * tm.shape[-1]
    M = np.zeros((N * bs, bs), dtype=complex)
    for i in range(N):
        try:
            M[i * bs:(i + 1) * bs] = np.linalg.inv(np.eye(bs) + tm[i].reshape(bs, bs))
        except np.linalg.LinAlgError:
            M[i * bs:(i + 1) * bs] = np.eye(bs)
    return M, bs


def solve_linear_system_precond(T, b, M_inv_blocks, block_size, method="bicgstab", tol=1e-5, maxiter=1000):
    """(I + T) x = b with Eigen's BiCGSTAB right-preconditioned by M_inv_blocks.
    Returns (x, iterations, relative residual)."""
    T = _c128(T)
    D = int(round(np.sqrt(T.size)))
    b = _c128(b).reshape(D)
    M = _c128(M_inv_blocks).reshape(D, block_size)
    x = np.empty(D, dtype=np.complex128)
    err = ctypes.c_double(0.0)
    meth = 1 if (getattr(method, "name", method) == "exact" or method == 1) else 0
    it = lib().orc_solve_linear_system_precond(D, _dp(T.view(np.float64)), _dp(b.view(np.float64)), meth,
                                               _dp(M.view(np.float64)), int(block_size), float(tol), int(maxiter),
                                               _dp(x.view(np.float64)), ctypes.byref(err))
    if it < 0:
        raise np.linalg.LinAlgError("singular interaction matrix")
    return x, it, err.value


def bicgstab_preconditioned(A, b, M_inv_blocks, block_size, maxiter=1000, tolerance=1e-5):
    """The reference's bicgstab_preconditioned_profiled (x0 = b, absolute tolerance).
    A includes the identity.  Returns (x, iters, residual)."""
    A = _c128(A)
    D = A.shape[0]
    b = _c128(b).reshape(D)
    M = _c128(M_inv_blocks).reshape(D, block_size)
    x = np.empty(D, dtype=np.complex128)
    err = ctypes.c_double(0.0)
    it = lib().orc_bicgstab_precond(D, _dp(A.view(np.float64)), _dp(b.view(np.float64)), _dp(M.view(np.float64)),
                                    int(block_size), int(maxiter), float(tolerance), _dp(x.view(np.float64)),
                                    ctypes.byref(err))
    return x, it, err.value


def gemv(A, x):
    A = _c128(A)
    D = A.shape[0]
    x = _c128(x).reshape(D)
    y = np.empty(D, dtype=np.complex128)
    lib().orc_gemv(D, _dp(A.view(np.float64)), _dp(x.view(np.float64)), _dp(y.view(np.float64)))
    return y


# ------------------------------------------------------ cross sections, forces --
def particle_cross_sections(p_scat, p_inc, p_src, k):
    """Per particle; returns (Cscat, Cabs, Cext), each [2*lmax] (cpp/src/flux.cpp:5-30)."""
    ps, pi, pr = (_c128(a).ravel() for a in (p_scat, p_inc, p_src))
    rmax = ps.size // 2
    lmax = int(-1 + (1 + rmax) ** 0.5)
    out = np.empty(6 * lmax, dtype=np.float64)
    lib().orc_particle_cross_sections(rmax, _dp(ps.view(np.float64)), _dp(pi.view(np.float64)),
                                      _dp(pr.view(np.float64)), float(np.real(k)), _dp(out))
    return out[: 2 * lmax].copy(), out[2 * lmax: 4 * lmax].copy(), out[4 * lmax:].copy()


def cluster_cross_sections(p_cluster, p_src, k):
    pc, pr = (_c128(a).ravel() for a in (p_cluster, p_src))
    rmax = pc.size // 2
    lmax = int(-1 + (1 + rmax) ** 0.5)
    out = np.empty(6 * lmax, dtype=np.float64)
    lib().orc_cluster_cross_sections(rmax, _dp(pc.view(np.float64)), _dp(pr.view(np.float64)), float(np.real(k)),
                                     _dp(out))
    return out[: 2 * lmax].copy(), out[2 * lmax: 4 * lmax].copy(), out[4 * lmax:].copy()


def force(p_scat, p_inc, k, eps_b, mu_b=1.0):
    ps, pi = _c128(p_scat).ravel(), _c128(p_inc).ravel()
    F = np.empty(3, dtype=np.float64)
    lib().orc_force(ps.size // 2, _dp(ps.view(np.float64)), _dp(pi.view(np.float64)), float(np.real(k)),
                    float(np.real(eps_b)), _dp(F))
    return F


def torque(p_scat, p_inc, k, eps_b, mu_b=1.0):
    ps, pi = _c128(p_scat).ravel(), _c128(p_inc).ravel()
    T = np.empty(3, dtype=np.float64)
    lib().orc_torque(ps.size // 2, _dp(ps.view(np.float64)), _dp(pi.view(np.float64)), float(np.real(k)),
                     float(np.real(eps_b)), _dp(T))
    return T


def force_all(p_scat_all, p_inc_all, k, eps_b, mu_b=1.0):
    N = np.asarray(p_scat_all).shape[0]
    ps, pi = _c128(p_scat_all).reshape(N, -1), _c128(p_inc_all).reshape(N, -1)
    F = np.empty((N, 3), dtype=np.float64)
    lib().orc_force_all(N, ps.shape[1] // 2, _dp(ps.view(np.float64)), _dp(pi.view(np.float64)),
                        float(np.real(k)), float(np.real(eps_b)), _dp(F))
    return F


def torque_all(p_scat_all, p_inc_all, k, eps_b, mu_b=1.0):
    N = np.asarray(p_scat_all).shape[0]
    ps, pi = _c128(p_scat_all).reshape(N, -1), _c128(p_inc_all).reshape(N, -1)
    T = np.empty((N, 3), dtype=np.float64)
    lib().orc_torque_all(N, ps.shape[1] // 2, _dp(ps.view(np.float64)), _dp(pi.view(np.float64)),
                         float(np.real(k)), float(np.real(eps_b)), _dp(T))
    return T


# -------------------------------------------------------------- VSH fields --
def Emn(m, n):
    out = np.empty(2, dtype=np.float64)
    lib().orc_Emn(int(m), int(n), _dp(out))
    return complex(out[0], out[1])


def vsh_electric(n, m, mode, rad, theta, phi, k):
    out = np.empty(3, dtype=np.complex128)
    lib().orc_vsh_electric(int(n), int(m), mode_value(mode), float(rad), float(theta), float(phi), float(k),
                           _dp(out.view(np.float64)))
    return out


def vsh_magnetic(n, m, mode, rad, theta, phi, k):
    out = np.empty(3, dtype=np.complex128)
    lib().orc_vsh_magnetic(int(n), int(m), mode_value(mode), float(rad), float(theta), float(phi), float(k),
                           _dp(out.view(np.float64)))
    return out


def expand_E_cluster(pos, p_expand, mode, x, y, z, k):
    """pos [N,3], p_expand [N, 2*rmax] -> E [Npts, 3] (cpp/src/vsh_functions.cpp:100-143)."""
    pos = _f64(pos).reshape(-1, 3)
    N = pos.shape[0]
    P = _c128(p_expand).reshape(N, -1)
    x, y, z = (_f64(np.ravel(a)) for a in (x, y, z))
    E = np.empty((x.size, 3), dtype=np.complex128)
    lib().orc_expand_E_cluster(N, P.shape[1] // 2, _dp(pos), _dp(P.view(np.float64)), mode_value(mode), x.size,
                               _dp(x), _dp(y), _dp(z), float(np.real(k)), _dp(E.view(np.float64)))
    return E


# ----------------------------------------------------------- decomposition --
def trapz(x, y):
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=complex)
    return complex(np.sum((y[1:] + y[:-1]) * (x[1:] - x[:-1]) / 2.0))


def trapz_2d(x, y, f):
    f = np.asarray(f, dtype=complex)
    z = np.array([trapz(x, f[:, i]) for i in range(len(y))])
    return trapz(y, z)


def integrate_phase(rhat, origin, k, rmax, theta, phi, p0):
    rhat = _f64(rhat)
    origin = _f64(origin).ravel()
    theta, phi = _f64(theta), _f64(phi)
    p0 = _c128(p0)
    out = np.empty((2, rmax), dtype=np.complex128)
    lib().orc_integrate_phase(_dp(rhat), _dp(origin), float(np.real(k)), int(rmax), theta.size, _dp(theta), phi.size,
                              _dp(phi), _dp(p0.view(np.float64)), _dp(out.view(np.float64)))
    return out

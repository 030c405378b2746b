"""Clusters of general particles given by their T-matrices.

Mirrors the solve of the reference's ``miepy.cluster`` (cluster.py:629-657): p_src
from the source, (I + T_agg) p_inc = p_src with the aggregate of
``particle_aggregate_tmatrix`` (interactions.cpp:417-462, block (i, j) = A_ij T_j),
p_scat = T p_inc (cluster.py:657, ``einsum("naibj,nbj->nai")``), then cross-sections
(flux.particle_cross_sections, cluster.py:407-421), forces and torques
(cluster.py:472-510).  The particle T-matrices are the caller's ([N, 2, rmax, 2,
rmax], the reference's layout): ``tmatrix_sphere`` for spheres, or T-matrices
computed elsewhere (the reference's EBCM particle classes, core-shell Mie) for other
particles.  On the GPU the packed translation blocks A are applied after each
particle's T-matrix (``gb_solve_batch_tmatrix``); the dense aggregate is formed only
for lmax > 8, beyond the packed solvers' order limit (``gb_particle_aggregate_dense``
then ``gb_solve_dense``).
"""

from __future__ import annotations

import types
import warnings

import numpy as np
import torch

from . import _native as nat
from .cluster import (DEFAULT_MAXITER, DEFAULT_TOL, EXACT_TOL, _method_is_exact, cross_sections, far_expansions,
                      sph_points, sphere_cluster, vec_to_sph)
from .engine import ClusterBatch, current_stream
from .materials import constant_material
from .mie import mie_coefficients
from .modes import lmax_to_rmax


def tmatrix_sphere(radius, wavelength, eps, eps_m, lmax, conducting=False):
    """T-matrix [2, rmax, 2, rmax] of a sphere (tmatrix/common.py:6-28): a_n on the
    electric and b_n on the magnetic diagonal, for every m of each n."""
    n_m = np.sqrt(complex(eps_m))
    k_b = 2 * np.pi * np.real(n_m) / wavelength
    ms, _ = mie_coefficients(np.atleast_1d(radius), np.atleast_1d(complex(eps)), np.ones(1, complex),
                             complex(eps_m), 1.0 + 0j, k_b, lmax, np.atleast_1d(conducting))
    rmax = lmax_to_rmax(lmax)
    T = np.zeros((2, rmax, 2, rmax), dtype=complex)
    r = 0
    for n in range(1, lmax + 1):
        for _m in range(-n, n + 1):
            T[0, r, 0, r] = ms[0, 0, n - 1]
            T[1, r, 1, r] = ms[0, 1, n - 1]
            r += 1
    return T


class sphere:
    """A sphere particle for ``cluster`` (particles/sphere.py): position, radius,
    material; its T-matrix from Mie theory."""

    def __init__(self, position, radius, material):
        self.position = np.asarray(position, dtype=float)
        self.radius = float(radius)
        self.material = material
        self.tmatrix = None

    def enclosed_radius(self):
        return self.radius

    def compute_tmatrix(self, lmax, wavelength, eps_m, **kwargs):
        metal = getattr(self.material, "name", None) == "metal"
        self.tmatrix = tmatrix_sphere(self.radius, wavelength, self.material.eps(wavelength), eps_m, lmax, metal)
        return self.tmatrix


class tmatrix_cluster:
    """GMT solve for N particles given by T-matrices [N, 2, rmax, 2, rmax].

    Keywords as the reference's cluster where they apply (source, wavelength, lmax,
    medium, interactions, method), plus precision ("fp64" default, "mixed", "fp32"),
    tol, maxiter, device, origin (of the cluster coefficients, default 0) and
    enclosed_radius ([N], the radius of each particle's circumscribing sphere, for
    the interior rule of the fields; none by default).
    """

    # cluster coefficients, per-multipole cluster cross-sections and far fields
    # depend only on positions, p_scat, the source and the medium: the sphere
    # cluster's GPU implementations (cluster.py:379-391, 616-627)
    solve_cluster_coefficients = sphere_cluster.solve_cluster_coefficients
    cross_sections_per_multipole = sphere_cluster.cross_sections_per_multipole
    _angular = sphere_cluster._angular

    def E_angular(self, theta, phi, radius=None, source=False):
        """Far-field E (theta, phi components) of the particles (cluster.py:349-362:
        the far expansions evaluated at radius, by default one wavelength 2 pi / k)."""
        return self._angular(theta, phi, 2 * np.pi / self.k_b if radius is None else radius, source, magnetic=False)

    def H_angular(self, theta, phi, radius=None, source=False):
        """Far-field H (theta, phi components) of the particles (cluster.py:364-377)."""
        return self._angular(theta, phi, 2 * np.pi / self.k_b if radius is None else radius, source, magnetic=True)

    def __init__(self, *, position, tmatrix, source, wavelength, lmax, medium=None, interactions=True, method=None,
                 precision="fp64", tol=None, maxiter=None, device=None, enclosed_radius=None, origin=None):
        self.position = np.asarray(np.atleast_2d(position), dtype=float)
        N = self.position.shape[0]
        self.Nparticles = N
        self.lmax = int(lmax)
        self.rmax = lmax_to_rmax(self.lmax)
        self.tmatrix = np.asarray(tmatrix, dtype=complex).reshape(N, 2, self.rmax, 2, self.rmax)
        self.source = source
        self.wavelength = wavelength
        self.medium = medium if medium is not None else constant_material(eps=1.0, mu=1.0)
        self.eps_b = complex(self.medium.eps(wavelength))
        self.mu_b = complex(self.medium.mu(wavelength))
        if self.eps_b.imag != 0 or self.mu_b.imag != 0:
            raise ValueError("medium must be non-absorbing")
        self.k_b = 2 * np.pi * np.real(np.sqrt(self.eps_b * self.mu_b)) / wavelength
        self.material_data = types.SimpleNamespace(k_b=self.k_b, eps_b=self.eps_b, mu_b=self.mu_b)
        self.origin = np.zeros(3) if origin is None else np.asarray(origin, dtype=float)
        self.p_cluster = None
        self.interactions, self.method, self.precision = interactions, method, precision
        self.tol, self.maxiter, self.device = tol, maxiter, device
        self.enclosed = np.zeros(N) if enclosed_radius is None else np.broadcast_to(
            np.asarray(enclosed_radius, dtype=float), (N,)).copy()
        self.solve()

    def _tolerance(self):
        if self.tol is not None:
            return float(self.tol)
        return EXACT_TOL if _method_is_exact(self.method) else DEFAULT_TOL

    def solve(self):
        N = self.Nparticles
        self.p_src = np.asarray(self.source.structure(self.position, self.k_b, self.lmax), dtype=complex)
        spec = dict(position=self.position, tmatrix=self.tmatrix, k=float(self.k_b), p_src=self.p_src)
        dense = self.interactions and N > 1 and self.lmax > 8   # the packed solvers take lmax <= 8
        prec = self.precision if self.interactions and not dense else "fp64"
        b = ClusterBatch([spec], R=1, precision=prec, device=self.device, packed=not dense)
        if dense:
            self._solve_dense(b)
        elif self.interactions and N > 1:
            tol = self._tolerance()
            b.assemble()
            b.solve(tol=tol, maxiter=self.maxiter or DEFAULT_MAXITER, inner_tol=min(1e-6, max(tol, 1e-7)),
                    max_refine=8)
            self.solver_status, self.solver_iterations = int(b.status[0]), int(b.iters[0])
            self.solver_residual = float(b.resid[0])
        else:   # no interactions: p_inc = p_src (cluster.py:648-650)
            b.x.copy_(b.b)
            self.solver_status, self.solver_iterations, self.solver_residual = 0, 0, 0.0
        b.epilogue(np.real(self.eps_b), source=True)
        view = lambda t: b.cluster_view(0, t)[..., 0].cpu().numpy()
        self.p_inc, self.p_scat = view(b.x), view(b.p_scat)
        L = self.lmax
        self._xs = b.xs[: N * 6 * L].view(N, 3, 2, L).cpu().numpy()
        self._F = b.F[: N * 3].view(N, 3).cpu().numpy()
        self._T = b.T[: N * 3].view(N, 3).cpu().numpy()
        self._batch = b

    def _solve_dense(self, b):
        """(I + T_agg) p_inc = p_src on the dense reference layout, as cluster.py:653-655
        with interactions.cpp:416-462: the translation blocks times each particle's
        T-matrix (gb_particle_aggregate_dense), then BiCGSTAB (gb_solve_dense) in FP64,
        the route of lmax > 8 whatever `precision` says (with a warning when it says
        otherwise)."""
        if self.precision != "fp64":
            warnings.warn(f"precision={self.precision!r} does not apply to T-matrix clusters of lmax > 8: their "
                          "dense operator is solved in FP64", stacklevel=3)
        L = nat.lib()
        dev, st = b.device, current_stream(b.device)
        N = self.Nparticles
        D = 2 * self.rmax * N
        ws = torch.empty(L.gb_particle_aggregate_workspace_size(N, self.lmax), dtype=torch.uint8, device=dev)
        T = torch.empty(D * D, dtype=torch.complex128, device=dev)
        nat.check(L.gb_particle_aggregate_dense(N, self.lmax, nat.ptr(b.pos), nat.ptr(b.tmat128), float(self.k_b),
                                                nat.ptr(ws), ws.numel(), nat.ptr(T), st), "particle aggregate")
        del ws
        need = L.gb_solve_dense_workspace_size(D, 1)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        status = np.zeros(1, np.int32)
        iters = np.zeros(1, np.int32)
        resid = np.zeros(1)
        rc = L.gb_solve_dense(D, 1, nat.ptr(T), nat.ptr(b.b), nat.ptr(b.x), self._tolerance(),
                              int(self.maxiter or DEFAULT_MAXITER), nat.ptr(ws), ws.numel(), status.ctypes.data,
                              iters.ctypes.data, resid.ctypes.data, st)
        if rc not in (nat.GB_OK, nat.GB_NOT_CONVERGED, nat.GB_BREAKDOWN, nat.GB_NAN):
            nat.check(rc, "dense solve")
        self.solver_status, self.solver_iterations, self.solver_residual = int(status[0]), int(iters[0]), float(resid[0])

    def cross_sections_per_multipole_of_particle(self, i):
        C = self._xs[i]
        return cross_sections(C[0].copy(), C[1].copy(), C[2].copy())

    def cross_sections_of_particle(self, i):
        return cross_sections(*[float(np.sum(c)) for c in self._xs[i]])

    def cross_sections(self):
        return cross_sections(*[float(v) for v in self._xs.sum(axis=(0, 2, 3))])

    def force(self):
        return self._F.copy()

    def torque(self):
        return self._T.copy()

    def force_on_particle(self, i):
        return self._F[i].copy()

    def torque_on_particle(self, i):
        return self._T[i].copy()

    # --------------------------------------------------------------- fields --
    def _field(self, x1, x2, x3, interior, source, mask, far, spherical, magnetic):
        """cluster.py:219-345: the outgoing expansions of every particle's p_scat
        plus the source.  Inside a particle's enclosed radius the reference evaluates
        its interior coefficients, which stay zero for general particles, so those
        points read 0 (interior=True) or are masked (mask=True).  Evaluated by the
        GPU near-field kernel (gb_near_field) with zero interior coefficients.
        spherical and far as for sphere_cluster (points about the cluster origin;
        far-field forms of the expansions, gb_far_field_expansions)."""
        x, y, z = sph_points(x1, x2, x3, self.origin, spherical)
        shape = x.shape
        pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
        dev = self._batch.device
        N, L = self.Nparticles, self.lmax
        hfac = -1j * np.sqrt(self.eps_b / self.mu_b) if magnetic else 1.0
        use_int = bool(interior and not mask and not far and np.any(self.enclosed > 0))
        if far:
            out = far_expansions(dev, self.position, self.p_scat, self.k_b, pts, magnetic, hfac)
        else:
            d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
            ps = d(self.p_scat, torch.complex128)
            zeros = torch.zeros_like(ps)
            ones = torch.ones(N, dtype=torch.complex128, device=dev)
            k_int = ones * self.k_b
            o = torch.empty((pts.shape[0], 3), dtype=torch.complex128, device=dev)
            pos, rad, P = d(self.position, torch.float64), d(self.enclosed, torch.float64), d(pts, torch.float64)
            nat.check(nat.lib().gb_near_field(N, L, nat.ptr(pos), nat.ptr(rad), nat.ptr(ps), nat.ptr(zeros),
                                              float(self.k_b), nat.ptr(k_int), pts.shape[0], nat.ptr(P), int(use_int),
                                              int(bool(magnetic)), float(np.real(hfac)), float(np.imag(hfac)),
                                              nat.ptr(ones), nat.ptr(o), current_stream(dev)), "near field")
            out = o.cpu().numpy()
        E = out.T.reshape((3,) + shape).copy()
        inside = np.zeros(shape, dtype=bool)
        for i in range(N):
            inside |= ((x - self.position[i, 0]) ** 2 + (y - self.position[i, 1]) ** 2
                       + (z - self.position[i, 2]) ** 2) < self.enclosed[i] ** 2
        if source:
            k = self.k_b
            S = (self.source.H_field(x, y, z, k, far=far) * (self.eps_b / self.mu_b) ** 0.5 if magnetic
                 else self.source.E_field(x, y, z, k, far=far))
            if use_int:
                S = np.where(inside[None], 0.0, S)
            E = E + S
        if mask and not far:
            E[:, inside] = 0
        if spherical:
            E = vec_to_sph(E, x2, x3)
        return E

    def E_field(self, x1, x2, x3, interior=True, source=True, mask=False, far=False, spherical=False):
        return self._field(x1, x2, x3, interior, source, mask, far, spherical, magnetic=False)

    def H_field(self, x1, x2, x3, interior=True, source=True, mask=False, far=False, spherical=False):
        return self._field(x1, x2, x3, interior, source, mask, far, spherical, magnetic=True)


class cluster(tmatrix_cluster):
    """The reference's ``miepy.cluster(particles=..., source, wavelength, lmax,
    medium, interactions, method)`` (cluster.py:16-112): each particle gives its
    position and ``compute_tmatrix(lmax, wavelength, eps_m)``; particles with equal
    ``_dict_key`` share one computed T-matrix, as the reference caches them."""

    def __init__(self, *, particles, source, wavelength, lmax, medium=None, origin=None, symmetry=None,
                 interface=None, interactions=True, method=None, **kw):
        if interface is not None:
            raise NotImplementedError("interface with cluster not supported (as the reference)")
        if symmetry is not None:
            raise NotImplementedError("symmetries with cluster not supported (as the reference)")
        self.particles = particles if isinstance(particles, list) else [particles]
        medium = medium if medium is not None else constant_material(eps=1.0, mu=1.0)
        eps_m = medium.eps(wavelength)
        rmax = lmax_to_rmax(lmax)
        T = np.empty((len(self.particles), 2, rmax, 2, rmax), dtype=complex)
        cache = {}
        for i, p in enumerate(self.particles):
            key = p._dict_key(wavelength) if hasattr(p, "_dict_key") else None
            if key is not None and key in cache:
                T[i] = cache[key]
                continue
            T[i] = p.compute_tmatrix(lmax, wavelength, eps_m)
            if key is not None:
                cache[key] = T[i]
        enclosed = [p.enclosed_radius() if hasattr(p, "enclosed_radius") else 0.0 for p in self.particles]
        enclosed = [0.0 if e is None else float(e) for e in enclosed]
        super().__init__(position=[p.position for p in self.particles], tmatrix=T, source=source,
                         wavelength=wavelength, lmax=lmax, medium=medium, interactions=interactions, method=method,
                         enclosed_radius=enclosed, origin=origin, **kw)

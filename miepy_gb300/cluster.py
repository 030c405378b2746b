"""sphere_cluster: the reference's Generalized Multiparticle Mie solver
(sphere_cluster.py:24-717) with its hot path on the GPU.

Same constructor, attributes (p_src, p_inc, p_scat, p_int as host numpy arrays of
shape [N, 2, rmax], mie_scat, mie_int, material_data, ...) and methods
(solve, cross_sections*, force*, torque*, E_field, H_field, update_position).
The interaction matrix is assembled in packed form, stays in HBM between
assembly and solve, and all observables come from the fused epilogue kernel.
"""

from __future__ import annotations

import enum
import warnings
from collections import namedtuple

import numpy as np
import torch

from . import _native as nat
from .engine import ClusterBatch, current_stream
from .materials import constant_material, material_struct
from .mie import mie_coefficients
from .modes import lmax_to_rmax

cross_sections = namedtuple("cross_sections", ["scattering", "absorption", "extinction"])


class solver(enum.Enum):
    """Solver choice (the reference's miepy.solver).  There is no LU on the GPU
    path: ``exact`` runs the same BiCGSTAB to a relative residual of 1e-14."""

    bicgstab = 0
    exact = 1


EXACT_TOL = 1e-14
DEFAULT_TOL = 1e-5      # the reference's BiCGSTAB tolerance (cpp/src/interactions.cpp:362)
DEFAULT_MAXITER = 1000  # cpp/src/interactions.cpp:363


def _atleast(x, length, dtype):
    a = np.asarray(x, dtype=dtype)
    if a.ndim == 0:
        a = np.full(length, a.item() if dtype is not object else x, dtype=dtype)
    return a


def _method_is_exact(method):
    if method is None:
        return False
    name = getattr(method, "name", None)
    return name == "exact" or method == 1 or str(method).endswith("exact")


def sph_points(x1, x2, x3, origin, spherical):
    """The points as Cartesian arrays: (r, theta, phi) about origin when spherical
    (coordinates.py:8-17), else (x, y, z) as given, broadcast to one shape."""
    x1, x2, x3 = np.broadcast_arrays(*(np.asarray(v, dtype=float) for v in (x1, x2, x3)))
    if not spherical:
        return x1, x2, x3
    o = np.asarray(origin, dtype=float)
    return (o[0] + x1 * np.sin(x2) * np.cos(x3), o[1] + x1 * np.sin(x2) * np.sin(x3), o[2] + x1 * np.cos(x2))


def vec_to_sph(F, theta, phi):
    """Cartesian field components -> (r, theta, phi) components at the given angles
    (vec_cart_to_sph, coordinates.py:71-89)."""
    theta, phi = np.broadcast_arrays(np.asarray(theta, float), np.asarray(phi, float))
    st, ct, sp, cp = np.sin(theta), np.cos(theta), np.sin(phi), np.cos(phi)
    basis = [(st * cp, st * sp, ct), (ct * cp, ct * sp, -st), (-sp, cp, 0.0 * theta)]
    return np.array([sum(b[c] * F[c] for c in range(3)) for b in basis])


def far_expansions(dev, position, p_scat, k, pts, magnetic, hfac):
    """Sum of every particle's outgoing expansion in its far-field form at pts
    [P, 3] (gb_far_field_expansions): [P, 3] complex on the host."""
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
    L = lmax_from_rmax(np.asarray(p_scat).shape[-1])
    out = torch.empty((pts.shape[0], 3), dtype=torch.complex128, device=dev)
    # every input stays referenced until the kernel has run
    pos, ps, P = d(position, torch.float64), d(p_scat, torch.complex128), d(pts, torch.float64)
    nat.check(nat.lib().gb_far_field_expansions(pos.shape[0], L, nat.ptr(pos), nat.ptr(ps), float(np.real(k)),
                                                pts.shape[0], nat.ptr(P), int(bool(magnetic)), float(np.real(hfac)),
                                                float(np.imag(hfac)), nat.ptr(out), current_stream(dev)), "far field")
    res = out.cpu().numpy()
    del pos, ps, P
    return res


def lmax_from_rmax(rmax):
    return int(round(np.sqrt(1 + rmax) - 1))


class sphere_cluster:
    """Solve Generalized Mie Theory for an N-sphere cluster on the GPU.

    Extra keywords beyond the reference's: ``precision`` ("fp64" default,
    "mixed", "fp32"), ``tol`` / ``maxiter`` (override the solver defaults),
    ``device``.
    """

    def __init__(self, *, position, radius, material, source, wavelength, lmax, medium=None, origin=None,
                 symmetry=None, interface=None, interactions=True, method=None, precision="fp64", tol=None,
                 maxiter=None, device=None):
        self.position = np.asarray(np.atleast_2d(position), dtype=float)
        N = self.position.shape[0]
        self.radius = _atleast(radius, N, float)
        mats = material if isinstance(material, (list, tuple, np.ndarray)) else [material] * N
        self.material = np.empty(N, dtype=object)
        for i, m in enumerate(mats):
            self.material[i] = m
        if not (self.position.shape[0] == self.radius.shape[0] == self.material.shape[0]):
            raise ValueError("The shapes of position, radius, and material do not match")
        self.Nparticles = N
        self.symmetry = symmetry
        self.interface = interface
        self.source = source
        self.wavelength = wavelength
        self.lmax = int(lmax)
        self.rmax = lmax_to_rmax(self.lmax)
        self.interactions = interactions
        self.method = method
        self.precision = precision
        self.tol = tol
        self.maxiter = maxiter
        self.device = device
        self.auto_origin = False
        if origin is None:
            self.origin = np.zeros(3)
        elif isinstance(origin, str) and origin == "auto":
            self.auto_origin = True
            self.origin = np.average(self.position, axis=0)
        else:
            self.origin = np.asarray(origin)
        if medium is None:
            self.medium = constant_material(eps=1.0, mu=1.0)
        else:
            self.medium = medium
            if np.imag(self.medium.eps(self.wavelength)) != 0 or np.imag(self.medium.mu(self.wavelength)) != 0:
                raise ValueError("medium must be non-absorbing")
        self.material_data = material_struct(self.material, self.medium, wavelength=self.wavelength)
        md = self.material_data
        conducting = np.array([getattr(m, "name", None) == "metal" for m in self.material])
        self.mie_scat, self.mie_int = mie_coefficients(self.radius, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b,
                                                       self.lmax, conducting)
        shape = [N, 2, self.rmax]
        self.p_inc = np.zeros(shape, dtype=complex)
        self.p_scat = np.zeros(shape, dtype=complex)
        self.p_int = np.zeros(shape, dtype=complex)
        self.p_src = np.zeros(shape, dtype=complex)
        self.p_cluster = None
        self._batch = None
        self.solver_status = None
        self.solver_iterations = None
        self.solver_residual = None
        self.solve()

    def __repr__(self):
        return (f"{self.__class__.__name__}:\n    Nparticles = {self.Nparticles}\n    source = {self.source}\n"
                f"    wavelength = {self.wavelength:.2e}\n    medium = {self.medium}\n    lmax = {self.lmax}\n"
                f"    origin = {self.origin}\n    precision = {self.precision}\n")

    # -------------------------------------------------------------- solving --
    def _tolerance(self):
        if self.tol is not None:
            return float(self.tol)
        return EXACT_TOL if _method_is_exact(self.method) else DEFAULT_TOL

    def solve(self, wavelength=None, source=None):
        if wavelength is not None or source is not None:
            raise NotImplementedError("re-solving at a new wavelength/source: build a new cluster")
        self.p_src[...] = self.source.structure(self.position, self.material_data.k_b, self.lmax)
        if self.interface is not None:   # sphere_cluster.py:683-685
            reflected = self.source.reflect(self.interface, self.medium, self.wavelength)
            self.p_src += reflected.structure(self.position, self.material_data.k_b, self.lmax)
        md = self.material_data
        spec = dict(position=self.position, mie_scat=self.mie_scat, mie_int=self.mie_int, k=float(np.real(md.k_b)),
                    p_src=self.p_src)
        prec = self.precision if self.interactions else "fp64"
        dense = self.interactions and (self.interface is not None or self.symmetry is not None or self.lmax > 8)
        b = ClusterBatch([spec], R=1, precision=prec, device=self.device, packed=not dense)
        if dense:
            self._solve_dense(b)   # (the packed solvers take lmax <= 8)
        elif self.interactions and self.Nparticles > 1:
            b.assemble()
            b.solve(tol=self._tolerance(), maxiter=self.maxiter or DEFAULT_MAXITER,
                    inner_tol=min(1e-6, max(self._tolerance(), 1e-7)), max_refine=8)
            self.solver_status = int(b.status[0])
            self.solver_iterations = int(b.iters[0])
            self.solver_residual = float(b.resid[0])
        else:
            # no interactions: p_inc = p_src (sphere_cluster.py:687-692)
            b.x.copy_(b.b)
            b.expand_only = True
            nat.check(nat.lib().gb_expand_mie_batch(b.nsys, b.sys, b.mie_off.ctypes.data, nat.ptr(b.mie_scat),
                                                    nat.ptr(b.tvec), current_stream(b.device)), "expand mie")
            self.solver_status, self.solver_iterations, self.solver_residual = 0, 0, 0.0
        b.epilogue(np.real(md.eps_b), source=True)
        self._batch = b
        view = lambda t: b.cluster_view(0, t)[..., 0]
        self.p_inc[...] = view(b.x).cpu().numpy()
        self.p_scat[...] = view(b.p_scat).cpu().numpy()
        self.p_int[...] = view(b.p_int).cpu().numpy()
        L = self.lmax
        self._xs = b.xs[: self.Nparticles * 6 * L].view(self.Nparticles, 3, 2, L).cpu().numpy()
        self._F = b.F[: self.Nparticles * 3].view(self.Nparticles, 3).cpu().numpy()
        self._T = b.T[: self.Nparticles * 3].view(self.Nparticles, 3).cpu().numpy()
        self._F_nosrc = self._T_nosrc = None

    def _solve_dense(self, b):
        """(I + T_agg - R) p_inc = p_src on the dense reference layout, as
        sphere_cluster.py:694-712: the aggregate T-matrix (gb_assemble_sphere_dense),
        or with a periodic symmetry the aggregate plus its lattice sums
        (gb_aggregate_periodic_dense), minus the interface's reflection matrix
        (gb_reflection_matrix_dense) when there is one; BiCGSTAB (gb_solve_dense),
        run to 1e-14 for solver.exact.  The interface and lattice operators are not
        symmetric in their pair blocks, and the packed solvers take lmax <= 8, so these
        are solved in FP64 whatever `precision` says (with a warning when it says
        otherwise)."""
        L = nat.lib()
        if self.precision != "fp64":
            warnings.warn(f"precision={self.precision!r} does not apply to clusters with an interface, a periodic "
                          "symmetry or lmax > 8: their dense operator is solved in FP64", stacklevel=3)
        dev, st = b.device, current_stream(b.device)
        md = self.material_data
        N, D = self.Nparticles, 2 * self.rmax * self.Nparticles
        k = float(np.real(md.k_b))
        nat.check(L.gb_expand_mie_batch(b.nsys, b.sys, b.mie_off.ctypes.data, nat.ptr(b.mie_scat), nat.ptr(b.tvec),
                                        st), "expand mie")
        T = torch.empty(D * D, dtype=torch.complex128, device=dev)
        if self.symmetry is not None:   # sphere_cluster.py:699-702
            from .backend import lattice_cells
            cells = lattice_cells(self.symmetry)
            kh = np.asarray(self.source.k_hat, dtype=float).reshape(3)
            d_cells = torch.from_numpy(cells).to(dev)
            nat.check(L.gb_aggregate_periodic_dense(N, self.lmax, nat.ptr(b.pos), nat.ptr(b.mie_scat), k,
                                                    nat.ptr(d_cells), cells.shape[0], float(kh[0]), float(kh[1]),
                                                    float(kh[2]), nat.ptr(T), st), "periodic aggregate")
        else:
            nat.check(L.gb_assemble_sphere_dense(N, self.lmax, nat.ptr(b.pos), nat.ptr(b.mie_scat), k, nat.ptr(T), st),
                      "dense assembly")
        if self.interface is not None:
            Rm = torch.empty_like(T)
            r0 = complex(self.interface.reflection_coefficients(0, self.wavelength, self.medium)[0])
            nat.check(L.gb_reflection_matrix_dense(N, self.lmax, nat.ptr(b.pos), nat.ptr(b.mie_scat), k, r0.real,
                                                   r0.imag, float(self.interface.z), nat.ptr(Rm), st),
                      "reflection matrix")
            T -= Rm
            del Rm
        # solver.exact is the same BiCGSTAB run to 1e-14 (_tolerance), as the plugin's exact branch
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

    def update_position(self, position):
        self.position = np.asarray(np.atleast_2d(position), dtype=float)
        self.p_cluster = None
        if self.auto_origin:
            self.origin = np.average(self.position, axis=0)
        self.solve()

    # --------------------------------------------------------- observables --
    def cross_sections_per_multipole_of_particle(self, i):
        C = self._xs[i]
        return cross_sections(C[0].copy(), C[1].copy(), C[2].copy())

    def cross_sections_of_particle(self, i):
        C = self.cross_sections_per_multipole_of_particle(i)
        return cross_sections(*[np.sum(A) for A in C])

    def cross_sections(self):
        Cs = Ca = Ce = 0
        for i in range(self.Nparticles):
            C = self.cross_sections_of_particle(i)
            Cs += C.scattering
            Ca += C.absorption
            Ce += C.extinction
        return cross_sections(Cs, Ca, Ce)

    # ------------------------------------------------- cluster coefficients --
    def solve_cluster_coefficients(self, lmax=None):
        """p_cluster [2, rmax(lmax)]: the particles' scattered fields re-expanded about
        the origin (sphere_cluster.py:650-661, vsh/cluster_coefficients.py:14-53), on the GPU."""
        lmax = self.lmax if lmax is None else int(lmax)
        dev = self._batch.device
        d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
        N = self.Nparticles
        L = nat.lib()
        ws = torch.empty(L.gb_cluster_coefficients_workspace_size(N, lmax), dtype=torch.uint8, device=dev)
        out = torch.empty(2 * lmax_to_rmax(lmax), dtype=torch.complex128, device=dev)
        pos = d(self.position, torch.float64)
        ps = d(self.p_scat, torch.complex128)
        origin = np.ascontiguousarray(np.asarray(self.origin, dtype=float))
        nat.check(L.gb_cluster_coefficients(N, self.lmax, nat.ptr(pos), nat.ptr(ps),
                                            float(np.real(self.material_data.k_b)), origin.ctypes.data, lmax,
                                            nat.ptr(out), nat.ptr(ws), ws.numel(), current_stream(dev)),
                  "cluster coefficients")
        self.p_cluster = out.cpu().numpy().reshape(2, lmax_to_rmax(lmax))
        return self.p_cluster

    def cross_sections_per_multipole(self, lmax=None):
        """Cluster cross-sections per multipole about the origin (sphere_cluster.py:428-440,
        flux.cluster_cross_sections flux.py:35-56): each [2, lmax]."""
        lmax = self.lmax if lmax is None else int(lmax)
        pc = self.solve_cluster_coefficients(lmax)
        k = float(np.real(self.material_data.k_b))
        p0 = self.source.structure(np.array([self.origin], dtype=float), k, lmax)[0]
        f = 4 * np.pi / k ** 2
        Cs = np.zeros((2, lmax))
        Ce = np.zeros((2, lmax))
        for r in range(lmax_to_rmax(lmax)):
            n = int(np.floor(np.sqrt(r + 1)))
            Cs[:, n - 1] += f * np.abs(pc[:, r]) ** 2
            Ce[:, n - 1] += f * np.real(np.conj(p0[:, r]) * pc[:, r])
        return cross_sections(Cs, Ce - Cs, Ce)

    def _angular(self, theta, phi, radius, source, magnetic):
        if source:
            raise NotImplementedError("source far fields (reflected sources) need substrate interfaces")
        md = self.material_data
        k = float(np.real(md.k_b))
        if radius is None:
            radius = 1e6 * 2 * np.pi / k
        th, ph, R = np.broadcast_arrays(np.asarray(theta, float), np.asarray(phi, float), np.asarray(radius, float))
        shape = th.shape
        dev = self._batch.device
        d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).reshape(-1)).to(dev, dtype=dt)
        pos = d(self.position, torch.float64)
        ps = d(self.p_scat, torch.complex128)
        Rt, Tt, Pt = d(R, torch.float64), d(th, torch.float64), d(ph, torch.float64)
        out = torch.empty((th.size, 2), dtype=torch.complex128, device=dev)
        hfac = -1j * np.sqrt(md.eps_b / md.mu_b) if magnetic else 1.0
        origin = np.ascontiguousarray(np.asarray(self.origin, dtype=float))
        nat.check(nat.lib().gb_far_field(self.Nparticles, self.lmax, nat.ptr(pos), nat.ptr(ps), k,
                                         origin.ctypes.data, th.size, nat.ptr(Rt), nat.ptr(Tt), nat.ptr(Pt),
                                         int(bool(magnetic)), float(np.real(hfac)), float(np.imag(hfac)),
                                         nat.ptr(out), current_stream(dev)), "far field")
        return out.cpu().numpy().T.reshape((2,) + shape)

    def E_angular(self, theta, phi, radius=None, source=False):
        """Far-field E (theta, phi components) of the particles (sphere_cluster.py:393-411)."""
        return self._angular(theta, phi, radius, source, magnetic=False)

    def H_angular(self, theta, phi, radius=None, source=False):
        """Far-field H (theta, phi components) of the particles (sphere_cluster.py:413-426)."""
        return self._angular(theta, phi, radius, source, magnetic=True)

    def _nosource(self):
        if self._F_nosrc is None:
            b = self._batch
            b.epilogue(np.real(self.material_data.eps_b), source=False, want_fields=False)
            N = self.Nparticles
            self._F_nosrc = b.F[: N * 3].view(N, 3).cpu().numpy()
            self._T_nosrc = b.T[: N * 3].view(N, 3).cpu().numpy()
        return self._F_nosrc, self._T_nosrc

    def force(self, source=True):
        return self._F.copy() if source else self._nosource()[0].copy()

    def torque(self, source=True):
        return self._T.copy() if source else self._nosource()[1].copy()

    def force_on_particle(self, i, source=True):
        return self.force(source)[i]

    def torque_on_particle(self, i, source=True):
        return self.torque(source)[i]

    # --------------------------------------------------------------- fields --
    def _field(self, x1, x2, x3, interior, source, mask, far, spherical, magnetic):
        """E or H at points (sphere_cluster.py:244-391).  spherical: the points are
        (r, theta, phi) about the cluster origin and the field is returned in
        spherical components there; far: every particle's outgoing expansion in its
        far-field form (gb_far_field_expansions), the source's far field, and no
        interior expansions or mask."""
        x, y, z = sph_points(x1, x2, x3, self.origin, spherical)
        shape = x.shape
        pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
        dev = self._batch.device
        md = self.material_data
        N, L = self.Nparticles, self.lmax
        d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
        pos = d(self.position, torch.float64)
        ps = d(self.p_scat, torch.complex128)
        hfac = -1j * np.sqrt(md.eps_b / md.mu_b) if magnetic else 1.0
        P = d(pts, torch.float64)
        out = torch.empty((pts.shape[0], 3), dtype=torch.complex128, device=dev)
        use_int = bool(interior and not mask and not far)
        if far:
            out = torch.from_numpy(far_expansions(dev, self.position, self.p_scat, md.k_b, pts, magnetic, hfac))
        else:
            rad = d(self.radius, torch.float64)
            pi_ = d(self.p_int, torch.complex128)
            k_int = d(2 * np.pi * np.asarray(md.n, complex) / self.wavelength, torch.complex128)
            hint = d(-1j * np.sqrt(np.asarray(md.eps, complex) / np.asarray(md.mu, complex)), torch.complex128)
            nat.check(nat.lib().gb_near_field(N, L, nat.ptr(pos), nat.ptr(rad), nat.ptr(ps), nat.ptr(pi_),
                                              float(np.real(md.k_b)), nat.ptr(k_int), pts.shape[0], nat.ptr(P),
                                              int(use_int), int(bool(magnetic)), float(np.real(hfac)),
                                              float(np.imag(hfac)), nat.ptr(hint), nat.ptr(out),
                                              current_stream(dev)), "near field")
        E = out.cpu().numpy().T.reshape((3,) + shape).copy()
        inside = np.zeros(shape, dtype=bool)
        for i in range(N):
            inside |= (x - self.position[i, 0]) ** 2 + (y - self.position[i, 1]) ** 2 + \
                (z - self.position[i, 2]) ** 2 < self.radius[i] ** 2
        if source:
            k = md.k_b
            srcs = [self.source]
            if self.interface is not None:   # sphere_cluster.py:279-283, 355-361
                srcs.append(self.source.reflect(self.interface, self.medium, self.wavelength))
            if not all(hasattr(s, "E_field") for s in srcs):
                raise NotImplementedError(f"{type(self.source).__name__} sources provide no field here; "
                                          "use source=False")
            S = sum(s.H_field(x, y, z, k, far=far) * (md.eps_b / md.mu_b) ** 0.5 if magnetic
                    else s.E_field(x, y, z, k, far=far) for s in srcs)
            if use_int:
                S = np.where(inside[None], 0.0, S)
            E = E + S
        if mask and not far:
            E[:, inside] = 0
        if spherical:   # components along the points' own (r, theta, phi) directions
            E = vec_to_sph(E, x2, x3)
        return E

    def E_field(self, x1, x2, x3, interior=True, source=True, mask=False, far=False, spherical=False):
        return self._field(x1, x2, x3, interior, source, mask, far, spherical, magnetic=False)

    def _field_from_particle(self, i, x, y, z, source, magnetic):
        """sphere_cluster.py:150-200: particle i's outgoing expansion of p_scat plus its
        regular (j_n, incident) expansion of p_inc (p_inc - p_src without the source),
        about its own centre, at every point.  Two launches of the GPU near-field
        kernel: exterior sums only, then the regular expansion alone (every point
        counts as inside a sphere of unbounded radius, with k_b as its wavenumber)."""
        x, y, z = np.broadcast_arrays(*(np.asarray(v, dtype=float) for v in (x, y, z)))
        shape = x.shape
        pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
        dev = self._batch.device
        md = self.material_data
        k = float(np.real(md.k_b))
        d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
        pos = d(self.position[i: i + 1], torch.float64)
        ps = d(self.p_scat[i: i + 1], torch.complex128)
        p_reg = self.p_inc[i] - (0 if source else self.p_src[i])
        pr = d(p_reg[None], torch.complex128)
        zeros = torch.zeros_like(ps)
        P = d(pts, torch.float64)
        hfac = complex(-1j * np.sqrt(md.eps_b / md.mu_b)) if magnetic else 1.0 + 0j
        k_reg = torch.full((1,), k, dtype=torch.complex128, device=dev)
        h_reg = torch.full((1,), hfac, dtype=torch.complex128, device=dev)
        big = torch.full((1,), 1e150, dtype=torch.float64, device=dev)
        L = nat.lib()
        outs = []
        for interior, cs, ci, rad in ((0, ps, zeros, big), (1, zeros, pr, big)):
            out = torch.empty((pts.shape[0], 3), dtype=torch.complex128, device=dev)
            nat.check(L.gb_near_field(1, self.lmax, nat.ptr(pos), nat.ptr(rad), nat.ptr(cs), nat.ptr(ci), k,
                                      nat.ptr(k_reg), pts.shape[0], nat.ptr(P), interior, int(bool(magnetic)),
                                      float(hfac.real), float(hfac.imag), nat.ptr(h_reg), nat.ptr(out),
                                      current_stream(dev)), "field from particle")
            outs.append(out)
        E = (outs[0] + outs[1]).cpu().numpy().T.reshape((3,) + shape)
        return E

    def E_field_from_particle(self, i, x, y, z, source=True):
        """Electric field of particle i's expansions (sphere_cluster.py:150-173)."""
        return self._field_from_particle(i, x, y, z, source, magnetic=False)

    def H_field_from_particle(self, i, x, y, z, source=True):
        """Magnetic field of particle i's expansions (sphere_cluster.py:175-200)."""
        return self._field_from_particle(i, x, y, z, source, magnetic=True)

    def H_field(self, x1, x2, x3, interior=True, source=True, mask=False, far=False, spherical=False):
        return self._field(x1, x2, x3, interior, source, mask, far, spherical, magnetic=True)

    def E_source(self, x1, x2, x3, far=False, spherical=False):
        return self.source.E_field(x1, x2, x3, self.material_data.k_b, far=far, spherical=spherical)

    def H_source(self, x1, x2, x3, far=False, spherical=False):
        md = self.material_data
        return (md.eps_b / md.mu_b) ** 0.5 * self.source.H_field(x1, x2, x3, md.k_b, far=far, spherical=spherical)

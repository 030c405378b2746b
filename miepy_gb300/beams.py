"""Beam sources: Gaussian beams and their expansion coefficients at the particles.

The decomposition follows the reference's far-field integral method:

* theta_cutoff / E0 / scalar_angular_spectrum of gaussian_beam
  (sources/common.py:10-52) and the polarised angular spectrum
  (sources/sources.py:188-195);
* integral_project_source_far (vsh/decomposition.py:284-325): on a 20 x 40
  (theta, phi) far-field grid over [pi - theta_c, pi] x [0, 2 pi], project the
  angular spectrum onto the ingoing far-field VSHs N_mn, M_mn (vsh/vsh_functions.py:
  81-109) to get p0[a, r, theta, phi];
* integrate_phase (cpp/src/decomposition.cpp:29-66) per particle: the 2-D
  trapezoid integral of p0 times exp(-i k rhat . x_i).

The per-(k, lmax) projection p0 is a small host computation (numpy, cached on the
beam as in the reference); the per-particle integrals, which dominate for many
particles, run on the GPU in one launch (gb_beam_project).
"""

from __future__ import annotations

import numpy as np
import torch
from scipy.constants import physical_constants
from scipy.special import erfc

from . import _native as nat
from .modes import lmax_to_rmax, mode_indices
from .rotation import rotate_expansion_coefficients, rotation_matrix
from .special import Emn, pi_func, tau_func
from .sources import sph_basis_vectors

Z0 = physical_constants["characteristic impedance of vacuum"][0]


def _trapz_weights(x):
    """Weights of the composite trapezoid rule on the nodes x."""
    x = np.asarray(x, float)
    w = np.zeros_like(x)
    d = np.diff(x)
    w[:-1] += d / 2
    w[1:] += d / 2
    return w


# ------------------------------------------------------------ quaternions --
# The unit quaternions the reference's beams use for directions (numpy-quaternion's
# from_spherical_coords, product, inverse and as_spherical_coords), as (w, x, y, z)
# arrays.
def _q_from_sph(theta, phi):   # exp(phi k / 2) exp(theta j / 2): Rz(phi) Ry(theta)
    theta, phi = np.broadcast_arrays(np.asarray(theta, float), np.asarray(phi, float))
    return np.array([np.cos(phi / 2) * np.cos(theta / 2), -np.sin(phi / 2) * np.sin(theta / 2),
                     np.cos(phi / 2) * np.sin(theta / 2), np.sin(phi / 2) * np.cos(theta / 2)])


def _q_mul(a, b):
    a1, b1, c1, d1 = a
    a2, b2, c2, d2 = b
    return np.array([a1 * a2 - b1 * b2 - c1 * c2 - d1 * d2, a1 * b2 + b1 * a2 + c1 * d2 - d1 * c2,
                     a1 * c2 - b1 * d2 + c1 * a2 + d1 * b2, a1 * d2 + b1 * c2 - c1 * b2 + d1 * a2])


def _q_inv(q):
    return np.array([q[0], -q[1], -q[2], -q[3]]) / np.sum(np.asarray(q) ** 2, axis=0)


def _q_to_sph(q):
    w, x, y, z = q
    return 2 * np.arctan2(np.sqrt(x ** 2 + y ** 2), np.sqrt(w ** 2 + z ** 2)), np.arctan2(z, w) + np.arctan2(-x, y)


def rotate_sph(theta, phi, quat):
    """Directions (theta, phi) rotated by quat (coordinates.py:157-170), with the
    reference's correction of phi where theta = 0."""
    theta, phi = np.broadcast_arrays(np.asarray(theta, float), np.asarray(phi, float))
    tq = np.broadcast_to(np.asarray(quat, float).reshape((4,) + (1,) * theta.ndim), (4,) + theta.shape)
    th_r, ph_r = _q_to_sph(_q_mul(tq, _q_from_sph(theta, phi)))
    ph_r = np.array(ph_r, dtype=float)
    ph_r[theta == 0] *= 2
    return np.asarray(th_r, dtype=float), ph_r


def _pinned_host(t):
    """A device tensor as a numpy copy, read through a pinned buffer on the current
    stream (one synchronisation of that stream only)."""
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t, non_blocking=True)
    torch.cuda.current_stream(t.device).synchronize()
    return h.numpy().copy()


class gaussian_beam:
    """Gaussian beam (sources/common.py:10-52).  A beam at (theta, phi) is the +z beam
    rotated by Rz(phi) Ry(theta) about its centre (sources/sources.py:164,
    sources/beams.py:168-200): particle positions are taken into the beam's frame,
    decomposed there on the GPU, and the coefficients rotated back (Wigner-D,
    miepy_gb300.rotation)."""

    def __init__(self, width, polarization, power=1, theta_max=np.pi / 2, phase=0, center=None, theta=0, phi=0,
                 standing=False):
        if standing:
            raise NotImplementedError("standing beams are not on the sphere-cluster path")
        self.width = width
        self.polarization = np.asarray(polarization, dtype=complex)
        self.polarization = self.polarization / np.linalg.norm(self.polarization)
        self.power = power
        self.theta_max = theta_max
        self.phase = phase
        self.center = np.zeros(3) if center is None else np.asarray(center, float)
        self.theta = theta
        self.phi = phi
        self.amplitude = 1
        self._cache = {}

    def __repr__(self):
        return (f"gaussian_beam(width={self.width}, polarization={self.polarization}, power={self.power}, "
                f"center={self.center}, theta={self.theta}, phi={self.phi})")

    # ---------------------------------------------------- angular spectrum --
    def E0(self, k):
        c = 0.5 * (k * self.width) ** 2
        if c < 700:
            U0 = np.sqrt(Z0 * self.power / (np.pi * (1 - np.sqrt(np.pi * c) * np.exp(c) * erfc(np.sqrt(c)))))
        else:
            U0 = np.sqrt(Z0 * self.power / (np.pi * (1 / (2 * c) - 3 / (4 * c ** 2) + 15 / (8 * c ** 3))))
        return U0

    def scalar_angular_spectrum(self, theta, phi, k):
        return np.exp(-((k * self.width * np.tan(theta) / 2) ** 2))

    def angular_spectrum(self, theta, phi, k):
        U = self.scalar_angular_spectrum(theta, phi, k)
        Ex = U * self.polarization[0]
        Ey = U * self.polarization[1]
        return np.array([-Ex * np.cos(phi) - Ey * np.sin(phi), -Ex * np.sin(phi) + Ey * np.cos(phi)], dtype=complex)

    def theta_cutoff(self, k, cutoff=1e-6, tol=None):
        arg = np.sqrt(-2 * np.log(cutoff)) / (k * self.width)
        theta_c = np.pi / 2 if arg >= 1 else np.arctan(arg)
        return min(self.theta_max, theta_c, np.pi / 2 - 1e-5)

    # ------------------------------------------------------- decomposition --
    def far_projection(self, k, lmax, sampling=20):
        """(rhat [G,3], w [G, 2*rmax] c128): the ingoing-VSH projection p0 of the
        angular spectrum on the far-field grid, times the trapezoid weights."""
        key = (float(k), int(lmax), int(sampling))
        if key in self._cache:
            return self._cache[key]
        theta_0 = np.pi - self.theta_cutoff(k)
        theta = np.linspace(theta_0, np.pi, sampling)
        phi = np.linspace(0, 2 * np.pi, 2 * sampling)
        THETA, PHI = np.meshgrid(theta, phi, indexing="ij")
        rad = 1
        rhat = sph_basis_vectors(THETA, PHI)[0]
        Esrc = self.angular_spectrum(THETA, PHI, k) * np.exp(-1j * k) / rad
        E0 = self.E0(k) * np.exp(1j * self.phase)
        rmax = lmax_to_rmax(lmax)
        p0 = np.zeros((2, rmax) + THETA.shape, dtype=complex)
        z = k * rad
        sin_t = np.sin(THETA)
        for r, n, m in mode_indices(lmax):
            factor = E0 * k ** 2 * 1j ** (2 - n) * np.abs(Emn(m, n)) / (4 * np.pi)
            zn = np.exp(-1j * (z - (n + 1) * np.pi / 2)) / z      # ingoing far-field radial factor
            tau = tau_func(n, m, THETA)
            pi_ = pi_func(n, m, THETA)
            eph = np.exp(1j * m * PHI)
            fN = -zn * eph                                        # ingoing N carries a minus sign
            N = np.array([1j * tau * fN, -pi_ * fN])
            fM = zn * eph
            M = np.array([1j * pi_ * fM, -tau * fM])
            p0[0, r] = 2 * factor * np.sum(Esrc * np.conjugate(N), axis=0) * sin_t * rad ** 2
            p0[1, r] = 2 * factor * np.sum(Esrc * np.conjugate(M), axis=0) * sin_t * rad ** 2
        wgt = _trapz_weights(theta)[:, None] * _trapz_weights(phi)[None, :]          # [T, P]
        w = (p0 * wgt).reshape(2 * rmax, -1).T                                      # [G, 2*rmax]
        out = (np.ascontiguousarray(rhat.reshape(3, -1).T), np.ascontiguousarray(w))
        self._cache[key] = out
        return out

    def structure_device(self, position, k, lmax, out=None, out_stride=1, device=None):
        """p_src [N, 2, rmax] computed on the GPU into ``out`` (a device complex128
        tensor; element (i, c) at (i*2*rmax + c) * out_stride) or a new tensor."""
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        pos = np.asarray(position, float).reshape(-1, 3) - self.center
        N = pos.shape[0]
        rmax = lmax_to_rmax(lmax)
        rhat, w = self.far_projection(k, lmax)
        # uploads from pinned copies (pageable uploads share the driver's staging path
        # with other streams' copies and can wait behind their kernels)
        d_pos, d_rhat, d_w = (torch.from_numpy(np.ascontiguousarray(a)).pin_memory().to(dev, non_blocking=True)
                              for a in (pos, rhat, w))
        if out is None:
            out = torch.empty(N * 2 * rmax, dtype=torch.complex128, device=dev)
            out_stride = 1
        nat.check(nat.lib().gb_beam_project(N, 2 * rmax, rhat.shape[0], nat.ptr(d_pos), nat.ptr(d_rhat),
                                            nat.ptr(d_w), float(k), nat.ptr(out), int(out_stride),
                                            torch.cuda.current_stream(dev).cuda_stream), "beam projection")
        # keep the inputs alive until the kernel has run
        out._beam_inputs = (d_pos, d_rhat, d_w)
        return out

    def reflect(self, interface, medium, wavelength):
        """The beam reflected by a planar interface (beams.py:202-203, 323-365)."""
        return reflected_beam(self, interface, wavelength, medium)

    @property
    def rotated(self):
        return self.theta != 0 or self.phi != 0

    def structure(self, position, k, lmax):
        """p_src [N, 2, rmax] (host numpy), computed on the GPU (and rotated on the
        host for a beam at (theta, phi) != 0)."""
        pos = np.asarray(position, float).reshape(-1, 3)
        N = pos.shape[0]
        if not self.rotated:
            out = self.structure_device(pos, k, lmax)
            return _pinned_host(out).reshape(N, 2, lmax_to_rmax(lmax))
        Rm = rotation_matrix(self.phi, self.theta)
        # the beam frame: R^T (pos - center); structure_device subtracts the centre itself
        pos_b = (pos - self.center) @ Rm + self.center
        p = _pinned_host(self.structure_device(pos_b, k, lmax)).reshape(N, 2, lmax_to_rmax(lmax))
        return rotate_expansion_coefficients(p, self.phi, self.theta)


class reflected_beam(gaussian_beam):
    """A Gaussian beam reflected by a planar interface (beams.py:323-365): the
    incident beam's centre mirrored in the interface, direction pi - theta, and the
    incident angular spectrum weighted by the Fresnel coefficients of each plane-wave
    component, mapped through the two beam frames."""

    def __init__(self, incident, interface, wavelength, medium):
        center = np.array(incident.center, dtype=float)
        center[2] += 2 * (interface.z - center[2])
        gaussian_beam.__init__(self, width=incident.width, polarization=incident.polarization, power=incident.power,
                               theta_max=incident.theta_max, phase=incident.phase, center=center,
                               theta=np.pi - incident.theta, phi=incident.phi)
        self.incident = incident
        self.interface = interface
        self.wavelength = wavelength
        self.medium = medium

    def angular_spectrum(self, theta, phi, k):
        th, ph = rotate_sph(np.asarray(theta, float) - np.pi, phi, _q_from_sph(self.theta, self.phi))
        th = np.where(th > np.pi / 2, np.pi - th, th)
        r_par, r_perp = self.interface.reflection_coefficients(th, self.wavelength, self.medium)
        th, ph = rotate_sph(th - np.pi, ph, _q_inv(_q_from_sph(self.incident.theta, self.incident.phi)))
        U = self.incident.angular_spectrum(th, ph, k)
        U[0] *= r_par
        U[1] *= r_perp
        return -U

    def E0(self, k):
        return self.incident.E0(k)

    def theta_cutoff(self, k, cutoff=1e-6, tol=None):
        return self.incident.theta_cutoff(k, cutoff, tol)

    def reflect(self, interface, medium, wavelength):
        raise NotImplementedError("a reflected beam is not reflected again")

"""Incident sources: their expansion coefficients p_src at the particles and
their fields.

plane_wave follows the reference's sources/plane_waves.py:10-156 (from_string,
E_field, H_field, structure); polarisation basis and normalisation as in
polarized_propagating_source (sources/sources.py:150-195).
"""

from __future__ import annotations

import numpy as np

from .modes import lmax_to_rmax, mode_indices
from .special import Emn, pi_func, tau_func


def sph_basis_vectors(theta, phi):
    r_hat = np.array([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)])
    theta_hat = np.array([np.cos(theta) * np.cos(phi), np.cos(theta) * np.sin(phi), -np.sin(theta)])
    phi_hat = np.array([-np.sin(phi), np.cos(phi), 0.0 * np.asarray(theta)])
    return r_hat, theta_hat, phi_hat


class plane_wave:
    def __init__(self, polarization, amplitude=1, phase=0, theta=0, phi=0, standing=False):
        if standing:
            raise NotImplementedError("standing plane waves are not on the sphere-cluster path")
        self.polarization = np.asarray(polarization, dtype=complex)
        self.polarization = self.polarization / np.linalg.norm(self.polarization)
        self.amplitude = amplitude
        self.phase = phase
        self.theta = theta
        self.phi = phi
        self.k_hat, self.n_tm, self.n_te = sph_basis_vectors(theta, phi)

    def __repr__(self):
        return f"plane_wave(polarization={self.polarization}, amplitude={self.amplitude}, theta={self.theta}, phi={self.phi})"

    def reflect(self, interface, medium, wavelength):
        """The plane wave reflected by a planar interface (sources/plane_waves.py:172-188):
        direction theta -> pi - theta, Fresnel-weighted polarisation, phase referred to z."""
        theta = np.pi - self.theta
        k = 2 * np.pi * medium.index(wavelength) / wavelength
        phase = self.phase - 2 * k * self.k_hat[2] * interface.z
        r_parallel, r_perp = interface.reflection_coefficients(self.theta, wavelength, medium)
        polarization = [r_parallel * self.polarization[0], r_perp * self.polarization[1]]
        amplitude = np.linalg.norm(polarization) * self.amplitude
        if amplitude == 0:
            polarization = self.polarization
        return plane_wave(polarization=polarization, theta=theta, phi=self.phi, amplitude=amplitude, phase=phase)

    @classmethod
    def from_string(cls, polarization, direction="z", amplitude=1, phase=0, standing=False):
        dirs = {"z": (0, 0), "+z": (0, 0), "-z": (np.pi, 0), "x": (np.pi / 2, 0), "+x": (np.pi / 2, 0),
                "-x": (np.pi / 2, np.pi), "y": (np.pi / 2, np.pi / 2), "+y": (np.pi / 2, np.pi / 2),
                "-y": (np.pi / 2, 3 * np.pi / 2)}
        if direction not in dirs:
            raise ValueError(f"'{direction}' is not a valid direction of propagation. Use one of "
                             "['x', 'y', 'z', '-x', '-y', '-z']")
        theta, phi = dirs[direction]
        if polarization == direction[-1]:
            raise ValueError("polarization cannot be the same as the direction of propagation")
        if polarization == "x":
            pol = [1, 0] if direction[-1] == "z" else [0, -1]
        elif polarization == "y":
            pol = [0, 1]
        elif polarization == "z":
            pol = [-1, 0]
        elif polarization == "rhc":
            pol = [1, 1j]
        elif polarization == "lhc":
            pol = [1, -1j]
        else:
            raise ValueError(f"'{polarization}' is not a valid polarization. Use one of ['x', 'y', 'z', 'rhc', 'lhc']")
        return cls(polarization=pol, theta=theta, phi=phi, amplitude=amplitude, phase=phase, standing=standing)

    def _amp(self, x1, x2, x3, k):
        return (self.amplitude * np.exp(1j * k * (self.k_hat[0] * x1 + self.k_hat[1] * x2 + self.k_hat[2] * x3))
                * np.exp(1j * self.phase))

    def E_field(self, x1, x2, x3, k, far=False, spherical=False):
        if spherical:
            raise NotImplementedError("spherical source fields are not on the sphere-cluster path")
        pol = self.n_tm * self.polarization[0] + self.n_te * self.polarization[1]
        return np.einsum("i...,...->i...", pol, self._amp(x1, x2, x3, k))

    def H_field(self, x1, x2, x3, k, far=False, spherical=False):
        if spherical:
            raise NotImplementedError("spherical source fields are not on the sphere-cluster path")
        pol = self.n_te * self.polarization[0] - self.n_tm * self.polarization[1]
        return np.einsum("i...,...->i...", pol, self._amp(x1, x2, x3, k))

    def field_vectors(self):
        """(k_hat, E polarisation vector, H polarisation vector, amplitude * e^{i phase}) for device evaluation."""
        polE = self.n_tm * self.polarization[0] + self.n_te * self.polarization[1]
        polH = self.n_te * self.polarization[0] - self.n_tm * self.polarization[1]
        return np.asarray(self.k_hat, float), polE, polH, self.amplitude * np.exp(1j * self.phase)

    def structure(self, position, k, lmax):
        """p_src [N, 2, rmax] (sources/plane_waves.py:126-156)."""
        position = np.asarray(position, dtype=float).reshape(-1, 3)
        rmax = lmax_to_rmax(lmax)
        pi_vals = np.empty(rmax)
        tau_vals = np.empty(rmax)
        emn_vals = np.empty(rmax)
        m_vals = np.empty(rmax, dtype=int)
        for r, n, m in mode_indices(lmax):
            pi_vals[r] = pi_func(n, m, self.theta)
            tau_vals[r] = tau_func(n, m, self.theta)
            emn_vals[r] = np.abs(Emn(m, n))
            m_vals[r] = m
        phases = k * (position @ self.k_hat) + self.phase
        f = self.amplitude * np.exp(1j * (phases[:, None] - m_vals * self.phi)) * emn_vals
        p_src = np.empty([position.shape[0], 2, rmax], dtype=complex)
        p_src[:, 0, :] = f * (tau_vals * self.polarization[0] - 1j * pi_vals * self.polarization[1])
        p_src[:, 1, :] = f * (pi_vals * self.polarization[0] - 1j * tau_vals * self.polarization[1])
        return p_src

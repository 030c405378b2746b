"""Planar interface (substrate) below or above a sphere cluster.

Mirrors ``miepy.interface`` (interface.py:6-37): an infinite plane at height z
between the medium and a material, with Fresnel coefficients.  A cluster built
with ``interface=`` adds the reflected source to its source coefficients and
subtracts the reflection matrix (``gb_reflection_matrix_dense``, the GPU
counterpart of interactions.cpp:464-512) from its aggregate T-matrix, as
sphere_cluster.py:679-710 does.
"""

from __future__ import annotations

import numpy as np


class interface:
    def __init__(self, material, z=0):
        self.material = material
        self.z = z

    def get_relative_index(self, wavelength, medium):
        eps_m = medium.eps(wavelength)
        eps = self.material.eps(wavelength)
        return np.sqrt(complex(eps / eps_m))

    def transmission_angle(self, theta, wavelength, medium):
        m = self.get_relative_index(wavelength, medium)
        return np.arcsin(np.sin(theta) / m)

    def reflection_coefficients(self, theta, wavelength, medium):
        """(r_parallel, r_perp) of the Fresnel equations (interface.py:16-22)."""
        m = self.get_relative_index(wavelength, medium)
        theta_t = self.transmission_angle(theta, wavelength, medium)
        r_parallel = (m * np.cos(theta) - np.cos(theta_t)) / (m * np.cos(theta) + np.cos(theta_t))
        r_perp = (np.cos(theta) - m * np.cos(theta_t)) / (np.cos(theta) + m * np.cos(theta_t))
        return r_parallel, r_perp

    def transmission_coefficients(self, theta, wavelength, medium):
        """(t_parallel, t_perp) of the Fresnel equations (interface.py:29-35)."""
        m = self.get_relative_index(wavelength, medium)
        theta_t = self.transmission_angle(theta, wavelength, medium)
        t_parallel = 2 * np.cos(theta) / (m * np.cos(theta) + np.cos(theta_t))
        t_perp = 2 * np.cos(theta) / (np.cos(theta) + m * np.cos(theta_t))
        return t_parallel, t_perp

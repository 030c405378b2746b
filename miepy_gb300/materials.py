"""Materials and per-wavelength material data (the reference's
material_functions/create.py:43-110 and material_struct.py:4-49)."""

from __future__ import annotations

import numpy as np

HC_EV_NM = 1239.84193   # h c in eV nm


class material:
    def __init__(self, name=None):
        self.name = name

    def eps(self, wavelength):
        raise NotImplementedError

    def mu(self, wavelength):
        raise NotImplementedError

    def index(self, wavelength):
        return np.sqrt(self.eps(wavelength) * self.mu(wavelength))

    def __repr__(self):
        return str(self.name)


class constant_material(material):
    """Constant eps and mu (``index`` sets eps = index**2)."""

    def __init__(self, eps=1.0, mu=1.0, index=None, name=None):
        super().__init__(name)
        self.eps_value = index ** 2 if index is not None else eps
        self.mu_value = mu

    def eps(self, wavelength):
        return np.full(np.shape(wavelength), self.eps_value)[()]

    def mu(self, wavelength):
        return np.full(np.shape(wavelength), self.mu_value)[()]

    def __repr__(self):
        return self.name if self.name else f"constant_material(eps={self.eps_value}, mu={self.mu_value})"


def dielectric(index=None, eps=1.0, mu=1.0, name=None):
    if index is not None:
        return constant_material(index=index, name=name)
    return constant_material(eps=eps, mu=mu, name=name)


class function_material(material):
    """eps (and mu) given as functions of the wavelength."""

    def __init__(self, eps_function, mu_function=None, name=None):
        super().__init__(name)
        self.eps_function = eps_function
        self.mu_function = mu_function if mu_function is not None else (lambda wavelength: 1.0)
        self.f_eps = np.vectorize(lambda w: self.eps_function(w))
        self.f_mu = np.vectorize(lambda w: self.mu_function(w))

    def eps(self, wavelength):
        return self.f_eps(wavelength)[()]

    def mu(self, wavelength):
        return self.f_mu(wavelength)[()]


def drude_material(eps_inf, omega_p_ev, gamma_ev, name=None):
    """Drude permittivity eps(w) = eps_inf - wp^2 / (w^2 + i g w), energies in eV."""

    def eps(wavelength):
        w = HC_EV_NM * 1e-9 / wavelength
        return eps_inf - omega_p_ev ** 2 / (w ** 2 + 1j * gamma_ev * w)

    return function_material(eps, name=name or f"drude({eps_inf}, {omega_p_ev} eV, {gamma_ev} eV)")


class materials:
    @staticmethod
    def vacuum():
        return constant_material(index=1, name="vacuum")

    @staticmethod
    def air():
        return constant_material(index=1, name="air")

    @staticmethod
    def water():
        return constant_material(index=1.33, name="water")

    @staticmethod
    def metal():
        return constant_material(eps=complex(1, 1e40), name="metal")


class material_struct:
    """eps, mu, n per particle and eps_b, mu_b, n_b, k_b of the medium at one wavelength."""

    def __init__(self, materials_, medium, wavelength=None):
        self.materials = list(materials_)
        self.medium = medium
        N = len(self.materials)
        self.eps = np.zeros(N, dtype=complex)
        self.mu = np.zeros(N, dtype=complex)
        self.n = np.zeros(N, dtype=complex)
        self.eps_b = self.mu_b = self.n_b = self.k_b = None
        self._wavelength = None
        self.wavelength = wavelength

    @property
    def wavelength(self):
        return self._wavelength

    @wavelength.setter
    def wavelength(self, value):
        self._wavelength = value
        if value is None:
            return
        self.eps_b = self.medium.eps(value)
        self.mu_b = self.medium.mu(value)
        self.n_b = (self.eps_b * self.mu_b) ** 0.5
        self.k_b = 2 * np.pi * self.n_b / value
        for i, m in enumerate(self.materials):
            self.eps[i] = m.eps(value)
            self.mu[i] = m.mu(value)
        self.n[...] = (self.eps * self.mu) ** 0.5

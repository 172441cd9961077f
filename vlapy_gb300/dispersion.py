"""Electron-plasma-wave dispersion root, used to set up runs (driver frequency,
expected Landau rate).  Host-side setup, as vlapy/diagnostics/z_function.py:
Z(z) = i sqrt(pi) w(z) from scipy.special.wofz, Z'(z) = -2 (1 + z Z(z)), and a
Newton root of 1 - chi Z'(z) with chi = (wp / (vth k))^2 / 2."""

from __future__ import annotations

import numpy as np
from scipy import optimize, special


def plasma_dispersion(value):
    return special.wofz(value) * np.sqrt(np.pi) * 1j


def plasma_dispersion_prime(value):
    return -2.0 * (1.0 + value * plasma_dispersion(value))


def get_roots_to_electrostatic_dispersion(wp_e, vth_e, k0, maxwellian_convention_factor=2.0,
                                          initial_root_guess=None):
    if initial_root_guess is None:
        initial_root_guess = np.sqrt(wp_e ** 2.0 + 3 * (k0 * vth_e) ** 2.0)
    chi_e = np.power((wp_e / (vth_e * k0)), 2.0) / maxwellian_convention_factor

    def epsilon(z):
        return 1.0 - chi_e * plasma_dispersion_prime(z)

    root = optimize.newton(epsilon, initial_root_guess)
    return root * k0 * vth_e * np.sqrt(maxwellian_convention_factor)

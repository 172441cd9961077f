"""Electron-plasma-wave dispersion root, used to set up runs (the driver
frequency of a driven wave, the expected Landau rate of an undriven one).

For a Maxwellian electron distribution of thermal speed vth and plasma
frequency wp, the electrostatic dielectric function at wavenumber k is

    eps(zeta) = 1 + (1 + zeta Z(zeta)) / (k lambda_D)^2,
    zeta = w / (s k vth),  lambda_D = vth / wp,

with s = sqrt(2) for f ~ exp(-v^2 / (2 vth^2)) and Z the plasma dispersion
function, Z(zeta) = i sqrt(pi) w(zeta) with w the Faddeeva function
(scipy.special.wofz).  Z obeys Z' = -2 (1 + zeta Z), so eps = 1 - c Z'(zeta)
with c = 1 / (s^2 (k lambda_D)^2), and eps' = -c Z'' with
Z'' = -2 (Z + zeta Z').

The root is found by Newton's method on zeta with this exact derivative,
started from the Bohm-Gross frequency sqrt(wp^2 + 3 k^2 vth^2) and stopped
after the first step smaller than 1e-12 |zeta|: convergence is quadratic, so
the error left after that step is at the rounding level of eps itself (four
to six iterations for the wavenumbers of these workloads).  The entry point keeps the
name and arguments of vlapy/diagnostics/z_function.py:26-50, which returns
the same root (its secant iteration stops at a 1.5e-8 tolerance, so the two
agree to about that).
"""

from __future__ import annotations

import math

from scipy import special

_SQRT_PI = math.sqrt(math.pi)


def z_function(zeta):
    """Plasma dispersion function Z(zeta) = i sqrt(pi) w(zeta)."""
    return 1j * _SQRT_PI * special.wofz(zeta)


def z_prime(zeta):
    """Z'(zeta) = -2 (1 + zeta Z(zeta))."""
    return -2.0 * (1.0 + zeta * z_function(zeta))


def _newton_zeta(c, zeta, max_iter=60):
    """Root of 1 - c Z'(zeta) by Newton's method with eps' = 2 c (Z + zeta Z')."""
    for _ in range(max_iter):
        z = z_function(zeta)
        zp = -2.0 * (1.0 + zeta * z)
        eps = 1.0 - c * zp
        deps = 2.0 * c * (z + zeta * zp)
        step = eps / deps
        zeta = zeta - step
        if abs(step) <= 1e-12 * abs(zeta):
            return zeta
    raise RuntimeError("dispersion root: Newton iteration did not converge")


def get_roots_to_electrostatic_dispersion(wp_e, vth_e, k0, maxwellian_convention_factor=2.0,
                                          initial_root_guess=None):
    """Complex frequency w (real part: the wave frequency, imaginary part: the
    Landau rate) of the electron plasma wave at wavenumber k0.  The
    convention factor is s^2 above (2 for exp(-v^2 / (2 vth^2))); an initial
    guess, if given, is a frequency."""
    s = math.sqrt(maxwellian_convention_factor)
    scale = k0 * vth_e * s  # w = scale * zeta
    w0 = initial_root_guess if initial_root_guess is not None else math.sqrt(wp_e ** 2 + 3.0 * (k0 * vth_e) ** 2)
    c = (wp_e / (vth_e * k0)) ** 2 / maxwellian_convention_factor
    zeta = _newton_zeta(c, complex(w0) / scale)
    return zeta * scale

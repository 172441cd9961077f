"""Grids, initial state and parameter dictionaries -- the setup side of a run.

Same names, arguments and results as vlapy/initializers.py.  These run once on
the host (as in the reference) and produce the NumPy arrays from which a plan
is built; the per-step arithmetic never runs here.
"""

from __future__ import annotations

import numpy as np

from . import dispersion


def initialize_distribution(nx, nv, vmax=6.0):
    """Unit-temperature Maxwellian, trapz-normalised per x
    (vlapy/initializers.py:29-53)."""
    f = np.zeros([nx, nv], dtype=np.float64)
    dv = 2.0 * vmax / nv
    vax = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    f[:] = np.exp(-(vax ** 2.0) / 2.0)[None, :]
    return f / np.trapezoid(f, dx=dv, axis=1)[:, None]


def initialize_velocity_quantities(vmax, nv):
    """dv, v, kv (vlapy/initializers.py:56-69)."""
    dv = 2 * vmax / nv
    v = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    kv = np.fft.fftfreq(v.size, d=dv) * 2.0 * np.pi
    return dv, v, kv


def initialize_spatial_quantities(xmin, xmax, nx):
    """dx, x, kx, one_over_kx with the zero mode set to 0
    (vlapy/initializers.py:72-89)."""
    dx = (xmax - xmin) / nx
    x = np.linspace(xmin + dx / 2.0, xmax - dx / 2.0, nx)
    kx = np.fft.fftfreq(x.size, d=dx) * 2.0 * np.pi
    one_over_kx = np.zeros_like(kx)
    one_over_kx[1:] = 1.0 / kx[1:]
    return dx, x, kx, one_over_kx


def make_default_params_dictionary():
    """Default parameter dictionary (vlapy/initializers.py:118-149) with the
    GB300 backend selected."""
    return {
        "nx": 32,
        "xmin": 0.0,
        "nv": 512,
        "vmax": 6.4,
        "nt": 500,
        "tmax": 80,
        "fokker-planck": {"type": "lb", "solver": "batched_tridiagonal"},
        "vlasov-poisson": {"time": "leapfrog", "vdfdx": "exponential",
                           "edfdv": "exponential", "poisson": "spectral"},
        "backend": {"core": "gb300", "precision": "fp64", "max_GB_for_device": int(1)},
        "a0": 4e-7,
    }


def specify_collisions_to_dict(log_nu_over_nu_ld, all_params_dict):
    """nu = |nu_ld| * 10**log_nu_over_nu_ld, or 0 (vlapy/initializers.py:152-167)."""
    if log_nu_over_nu_ld is None:
        all_params_dict["nu"] = 0.0
    else:
        all_params_dict["nu"] = np.abs(all_params_dict["nu_ld"]) * 10 ** log_nu_over_nu_ld
    return all_params_dict


def specify_epw_params_to_dict(k0, all_params_dict):
    """EPW frequency, Landau rate, box size and phase velocity from the
    dispersion root (vlapy/initializers.py:170-189)."""
    root = dispersion.get_roots_to_electrostatic_dispersion(wp_e=1.0, vth_e=1.0, k0=k0)
    all_params_dict["w_epw"] = np.real(root)
    all_params_dict["nu_ld"] = np.imag(root)
    all_params_dict["xmax"] = 2.0 * np.pi / k0
    all_params_dict["v_ph"] = all_params_dict["w_epw"] / k0
    return all_params_dict

"""Charge density and spectral Poisson solve (mirror of vlapy/core/field.py).

Inputs and outputs are CUDA float64 tensors.  The FP64 kernels sum the
density with NumPy's pairwise tree, so n(x) matches np.trapz bit for bit for
equal f, and the Poisson solve handles any nx (FFT for powers of two, a
direct DFT otherwise).
"""

from __future__ import annotations

import torch

from ._plans import as_device, aux_plan, plan_for


def compute_charges(f, dv):
    """n(x) = trapz_v f (vlapy/core/field.py:27-36)."""
    f = as_device(f)
    nx, nv = f.shape
    out = torch.empty(nx, dtype=torch.float64, device=f.device)
    return aux_plan(nx, nv, dv).charge_density(f, out)


def __fft_solve__(net_charge_density, one_over_kx):
    """E = Re IFFT(i/kx FFT(rho)) (vlapy/core/field.py:39-49)."""
    rho = as_device(net_charge_density)
    nx = rho.shape[0]
    out = torch.empty(nx, dtype=torch.float64, device=rho.device)
    return aux_plan(nx, 2, 1.0, one_over_kx).poisson(rho, out)


def solve_for_field(charge_density, one_over_kx):
    """Field of 1 - n (vlapy/core/field.py:52-63)."""
    return __fft_solve__(1.0 - as_device(charge_density), one_over_kx)


def get_spectral_solver(plan):
    """driver + self field (vlapy/core/field.py:66-88)."""

    def solve_total_electric_field(driver_field, f):
        f = as_device(f)
        out = torch.empty(f.shape[0], dtype=torch.float64, device=f.device)
        drv = None if driver_field is None else as_device(driver_field)
        return plan.field_solve(f, drv, out)

    return solve_total_electric_field


def get_field_solver(stuff_for_time_loop, field_solver_implementation="spectral", all_params=None):
    """vlapy/core/field.py:91-107."""
    if field_solver_implementation == "spectral":
        return get_spectral_solver(plan_for(stuff_for_time_loop, all_params))
    raise NotImplementedError

"""Advection operators (mirror of vlapy/core/vlasov.py).

The closures take and return CUDA float64 tensors f[nx, nv]; the arithmetic
runs in the kernels of libvlagpu.so: shared-memory FFTs for the exponential
integrators, spline kernels for the semi-Lagrangian steps and a stencil
kernel for the centred difference.  Like the reference's closures they are
functional: the input tensor is left unchanged.
"""

from __future__ import annotations

import torch

from ._plans import as_device, plan_for, precision_of


def get_vdfdx_exponential(plan):
    """x-advection by the exponential integrator (vlapy/core/vlasov.py:83-110)."""

    def step_vdfdx_exponential(f, dt):
        out = as_device(f).clone()
        return plan.vdfdx(out, dt)

    return step_vdfdx_exponential


def get_edfdv_exponential(plan):
    """v-advection by the exponential integrator (vlapy/core/vlasov.py:113-140)."""

    def step_edfdv_exponential(f, e, dt):
        out = as_device(f).clone()
        return plan.edfdv(out, as_device(e), dt)

    return step_edfdv_exponential


def get_vdfdx_sl(plan):
    """Backward semi-Lagrangian x-advection (vlapy/core/vlasov.py:42-80): the
    not-a-knot cubic spline of each v column over the x grid extended by one
    periodic cell at each end, evaluated at x - v dt."""

    def update_spatial_adv_sl(f, dt):
        f = as_device(f)
        return plan.vdfdx_sl(f, torch.empty_like(f), dt)

    return update_spatial_adv_sl


def get_edfdv_sl(plan):
    """Backward semi-Lagrangian v-advection (vlapy/core/vlasov.py:168-210):
    the spline of each x row over the extended v grid, evaluated at v - e dt."""

    def update_velocity_adv_sl(f, e, dt):
        f = as_device(f)
        return plan.edfdv_sl(f, as_device(e), torch.empty_like(f), dt)

    return update_velocity_adv_sl


def get_edfdv_center_differenced(plan):
    """f - e df/dv dt with numpy.gradient's second-order stencils
    (vlapy/core/vlasov.py:143-165)."""

    def step_edfdv_center_difference(f, e, dt):
        f = as_device(f)
        return plan.edfdv_cd2(f, as_device(e), torch.empty_like(f), dt)

    return step_edfdv_center_difference


def _fp64_plan(stuff_for_time_loop, all_params, name):
    if precision_of(all_params) != "fp64":
        raise NotImplementedError(name + " is implemented in the fp64 precision mode only on GB300")
    return plan_for(stuff_for_time_loop, all_params)


def get_vdfdx(stuff_for_time_loop, vdfdx_implementation="exponential", all_params=None):
    """vlapy/core/vlasov.py:213-235."""
    if vdfdx_implementation == "exponential":
        return get_vdfdx_exponential(plan_for(stuff_for_time_loop, all_params))
    if vdfdx_implementation == "sl":
        return get_vdfdx_sl(_fp64_plan(stuff_for_time_loop, all_params, "v df/dx: <sl>"))
    raise NotImplementedError(
        "v df/dx: <" + vdfdx_implementation + "> has not yet been implemented on GB300")


def get_edfdv(stuff_for_time_loop, edfdv_implementation="exponential", all_params=None):
    """vlapy/core/vlasov.py:238-260."""
    if edfdv_implementation == "exponential":
        return get_edfdv_exponential(plan_for(stuff_for_time_loop, all_params))
    if edfdv_implementation == "cd2":
        return get_edfdv_center_differenced(_fp64_plan(stuff_for_time_loop, all_params, "e df/dv: <cd2>"))
    if edfdv_implementation == "sl":
        return get_edfdv_sl(_fp64_plan(stuff_for_time_loop, all_params, "e df/dv: <sl>"))
    raise NotImplementedError(
        "e df/dv: <" + edfdv_implementation + "> has not yet been implemented on GB300")

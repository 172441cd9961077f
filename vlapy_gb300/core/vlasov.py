"""Advection operators (mirror of vlapy/core/vlasov.py).

The closures take and return CUDA float64 tensors f[nx, nv]; the arithmetic
runs in the shared-memory FFT kernels of libvlagpu.so.  Like the reference's
closures they are functional: the input tensor is left unchanged.
"""

from __future__ import annotations

from ._plans import as_device, plan_for


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


def get_vdfdx(stuff_for_time_loop, vdfdx_implementation="exponential", all_params=None):
    """vlapy/core/vlasov.py:213-235."""
    if vdfdx_implementation == "exponential":
        return get_vdfdx_exponential(plan_for(stuff_for_time_loop, all_params))
    raise NotImplementedError(
        "v df/dx: <" + vdfdx_implementation + "> has not yet been implemented on GB300")


def get_edfdv(stuff_for_time_loop, edfdv_implementation="exponential", all_params=None):
    """vlapy/core/vlasov.py:238-260."""
    if edfdv_implementation == "exponential":
        return get_edfdv_exponential(plan_for(stuff_for_time_loop, all_params))
    raise NotImplementedError(
        "e df/dv: <" + edfdv_implementation + "> has not yet been implemented on GB300")

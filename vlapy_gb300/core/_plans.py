"""Plans built from the reference's stuff_for_time_loop dictionary and cached
on it, so the closure factories of vlasov/field/step share one device plan."""

from __future__ import annotations

import numpy as np
import torch

from ..field_driver import PulseDriver
from ..plan import Plan

_KEY = "_vlagpu_plans"
_AUX = {}


def precision_of(all_params) -> str:
    if not all_params:
        return "fp64"
    return all_params.get("backend", {}).get("precision", "fp64")


def collision_name(all_params) -> str:
    if not all_params or all_params.get("nu", 0.0) == 0.0:
        return "none"
    fp = all_params.get("fokker-planck", {})
    return fp.get("type", "lb")


def plan_for(stuff: dict, all_params=None, collision=None, integrator=None) -> Plan:
    collision = collision_name(all_params) if collision is None else collision
    if integrator is None:
        integrator = (all_params or {}).get("vlasov-poisson", {}).get("time", "leapfrog")
    precision = precision_of(all_params)
    drv = stuff.get("driver_function")
    pulses = drv.pulses if isinstance(drv, PulseDriver) else []
    key = (collision, integrator, precision, float(stuff.get("dt", 0.0)), float(stuff.get("nu", 0.0)),
           id(drv))
    cache = stuff.setdefault(_KEY, {})
    if key in cache:
        return cache[key]
    nx, nv = int(stuff["nx"]), int(stuff["nv"])
    dv = float(stuff["dv"])
    v = np.asarray(stuff["v"], dtype=np.float64)
    x = np.asarray(stuff.get("x", np.zeros(nx)), dtype=np.float64)
    kx = np.asarray(stuff.get("kx", np.zeros(nx)), dtype=np.float64)
    kv = np.asarray(stuff.get("kv", np.fft.fftfreq(nv, d=dv) * 2.0 * np.pi), dtype=np.float64)
    inv = np.asarray(stuff.get("one_over_kx", np.zeros(nx)), dtype=np.float64)
    dx = float(x[1] - x[0]) if nx > 1 else 0.0
    f_bg = None
    if precision == "fp32-deltaf":
        # the fixed background of the delta-f state: the x-average of the initial f
        f_bg = background_of(stuff["f"])
    p = Plan(nx, nv, x, v, kx, kv, inv, dx, dv, dt=float(stuff.get("dt", 0.0)),
             nu=float(stuff.get("nu", 0.0)), collision=collision, integrator=integrator,
             pulses=pulses, precision=precision, f_background=f_bg)
    cache[key] = p
    return p


def background_of(f) -> np.ndarray:
    """x-average of a distribution function (host float64)."""
    if isinstance(f, torch.Tensor):
        f = f.detach().cpu().numpy()
    return np.asarray(f, dtype=np.float64).mean(axis=0)


def to_deviation(plan, f):
    """FP32 deviation g = f - f0 of a plan in the delta-f mode (CUDA tensor)."""
    f0 = torch.as_tensor(plan._fbg, device="cuda")
    return (as_device(f) - f0[None, :]).to(torch.float32).contiguous()


def from_deviation(plan, g, out=None):
    """f = g + f0 as float64 (into out if given: one pass, no temporary)."""
    f0 = torch.as_tensor(plan._fbg, device="cuda")
    if out is not None:
        return torch.add(g, f0[None, :], out=out)
    return g.to(torch.float64) + f0[None, :]


_RESIDENT = "_g"


def resident_deviation(plan, temp_storage):
    """The FP32 deviation g = f - f0 of temp_storage["f"], kept with
    temp_storage between calls.  It is reused while temp_storage["f"] is the
    tensor that publish_deviation last wrote and nothing has written to it
    since (its version counter is unchanged); otherwise it is formed again
    from f, so a caller that replaces or edits f restarts from its f."""
    f = temp_storage["f"]
    held = temp_storage.get(_RESIDENT)
    if held is not None and isinstance(f, torch.Tensor):
        g, f_ref, version = held
        if f_ref is f and f._version == version:
            return g
    g = to_deviation(plan, f)
    if isinstance(f, torch.Tensor):
        temp_storage[_RESIDENT] = (g, f, f._version)
    return g


def publish_deviation(plan, temp_storage, g):
    """Write f = g + f0 into temp_storage["f"] (a float64 CUDA tensor, made
    one if it is not) and mark g as its resident deviation."""
    f = temp_storage["f"]
    if not (isinstance(f, torch.Tensor) and f.is_cuda and f.dtype == torch.float64 and f.is_contiguous()):
        f = temp_storage["f"] = torch.empty(g.shape, dtype=torch.float64, device=g.device)
    from_deviation(plan, g, out=f)
    temp_storage[_RESIDENT] = (g, f, f._version)
    return f


def aux_plan(nx: int, nv: int, dv: float, one_over_kx=None) -> Plan:
    """Plan for the stand-alone field functions (compute_charges,
    solve_for_field), keyed by the grid it needs."""
    inv = np.zeros(nx) if one_over_kx is None else np.asarray(one_over_kx, dtype=np.float64)
    key = (nx, nv, float(dv), inv.tobytes())
    if key not in _AUX:
        v = np.linspace(-1.0, 1.0, nv)
        _AUX[key] = Plan(nx, nv, np.zeros(nx), v, np.zeros(nx), np.zeros(nv), inv, 1.0, dv)
    return _AUX[key]


def as_device(a, dtype=torch.float64):
    """A CUDA tensor for a, copying host data (NumPy or CPU tensor) if needed."""
    if isinstance(a, torch.Tensor):
        if a.is_cuda and a.dtype == dtype and a.is_contiguous():
            return a
        return a.to(device="cuda", dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")

"""Step assembly (mirror of vlapy/core/step.py).

``get_timestep`` returns the per-step closure of the reference,
``timestep(temp_storage, i) -> (temp_storage, i)``, over a temp_storage dict
of CUDA tensors.  With a pulse (or no) driver the whole step -- VP step, FP
step and storage step -- is one call into libvlagpu (vg_run_steps); with an
arbitrary Python driver closure the step is composed from the operator
closures instead, evaluating the closure on the host at each sub-step time
exactly as the reference does.
"""

from __future__ import annotations

import torch

from ..field_driver import PulseDriver
from ..plan import history_struct
from . import collisions, field, vlasov, vlasov_poisson
from ._plans import as_device, plan_for, publish_deviation, resident_deviation


def get_vlasov_poisson_step(all_params, stuff_for_time_loop):
    """VP step from the chosen sub-operators (vlapy/core/step.py:29-67)."""
    vp = all_params["vlasov-poisson"]
    vdfdx = vlasov.get_vdfdx(stuff_for_time_loop, vp["vdfdx"], all_params)
    edfdv = vlasov.get_edfdv(stuff_for_time_loop, vp["edfdv"], all_params)
    solver = field.get_field_solver(stuff_for_time_loop, vp["poisson"], all_params)
    return vlasov_poisson.get_time_integrator(vp["time"], vdfdx, edfdv, solver, stuff_for_time_loop)


def get_collision_step(stuff_for_time_loop, all_params):
    """Identity when nu == 0, else the implicit FP solve on the device
    (vlapy/core/step.py:70-113)."""
    if all_params["nu"] == 0.0:
        def take_collision_step(f):
            return f
    elif all_params["nu"] > 0.0:
        collisions.check_names(all_params["fokker-planck"])
        plan = plan_for(stuff_for_time_loop, all_params, collision=all_params["fokker-planck"]["type"])

        def take_collision_step(f):
            out = as_device(f).clone()
            return plan.collision_step(out)
    else:
        raise NotImplementedError
    return take_collision_step


def n_modes_of(store_f_rule):
    """Modes the reference computes per step: it slices len(rule_dict)
    x-Fourier modes (vlapy/core/step.py:130-135) -- the number of keys of the
    rule dict, which equals len(rule["space"]) for the two-key rule of the
    LandauDamping diagnostic -- and broadcasts them into the len(space) slots
    of stored_f.  None means the store-all rule."""
    if store_f_rule["space"] == "all":
        return None
    if store_f_rule["space"][0] == "k0":
        return len(store_f_rule)
    raise NotImplementedError


def get_storage_step(stuff_for_time_loop, all_params=None):
    """Storage step (vlapy/core/step.py:231-283): stored_f, eight fields and
    seven series, all written on the device."""
    plan = plan_for(stuff_for_time_loop, all_params)
    n_modes = n_modes_of(stuff_for_time_loop["rules_to_store_f"])

    def storage_step(temp_storage, e, de, f, i):
        hist = history_struct(temp_storage, plan.nx, n_modes)
        plan.storage_step(f, e, de, hist, i)
        temp_storage["e"] = e
        temp_storage["f"] = f
        return temp_storage

    return storage_step


def _device_batches(temp_storage):
    for k in ("time_batch", "driver_array_batch"):
        if k in temp_storage:
            temp_storage[k] = as_device(temp_storage[k])


def get_timestep(all_params, stuff_for_time_loop):
    """One full step (vlapy/core/step.py:286-328)."""
    drv = stuff_for_time_loop.get("driver_function")
    fused = drv is None or isinstance(drv, PulseDriver)
    vp = all_params["vlasov-poisson"]
    for name, impl in (("vdfdx", "exponential"), ("edfdv", "exponential"), ("poisson", "spectral")):
        if vp[name] != impl:
            fused = False
    if all_params.get("nu", 0.0) > 0.0:
        collisions.check_names(all_params["fokker-planck"])

    if fused:
        plan = plan_for(stuff_for_time_loop, all_params)
        n_modes = n_modes_of(stuff_for_time_loop["rules_to_store_f"])

        def timestep(temp_storage, i):
            _device_batches(temp_storage)
            f, e = temp_storage["f"], temp_storage["e"]
            hist = history_struct(temp_storage, plan.nx, n_modes)
            if plan.precision == "fp32-deltaf":
                # the delta-f state stays resident in FP32 between calls; f is
                # refreshed from it after the step
                g = resident_deviation(plan, temp_storage)
                plan.run_steps(g, e, hist, temp_storage["time_batch"], temp_storage["driver_array_batch"],
                               i, 1, use_graph=False)
                publish_deviation(plan, temp_storage, g)
            else:
                plan.run_steps(f, e, hist, temp_storage["time_batch"], temp_storage["driver_array_batch"],
                               i, 1, use_graph=False)
            return temp_storage, i

        timestep.plan = plan
        return timestep

    vp_step = get_vlasov_poisson_step(all_params, stuff_for_time_loop)
    fp_step = get_collision_step(stuff_for_time_loop, all_params)
    storage_step = get_storage_step(stuff_for_time_loop, all_params)

    def timestep(temp_storage, i):
        _device_batches(temp_storage)
        e = temp_storage["e"]
        f = temp_storage["f"]
        t = float(temp_storage["time_batch"][i])
        de = temp_storage["driver_array_batch"][i]
        e, f = vp_step(e=e, f=f, t=t)
        f = fp_step(f=f)
        return storage_step(temp_storage, e, de, f, i), i

    return timestep


__all__ = ["get_timestep", "get_collision_step", "get_storage_step", "get_vlasov_poisson_step",
           "n_modes_of", "torch"]

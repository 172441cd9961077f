"""Inner loop over a batch of steps (mirror of vlapy/outer_loop.py).

Select it with ``all_params["backend"]["core"] = "gb300"``.  The sim_config
dictionary has the reference's keys and shapes (vlapy/outer_loop.py:190-215)
with CUDA tensors as values; the inner loop runs every step of the batch as
one captured CUDA graph of the fused step kernels, then does the post-batch
series update on the device.
"""

from __future__ import annotations

import numpy as np
import torch

from . import field_driver, initializers
from .core import step
from .core._plans import as_device, plan_for, publish_deviation, resident_deviation
from .field_driver import PulseDriver
from .plan import history_struct, require_cuda

BACKENDS = ("gb300", "cuda")


def _check_backend(all_params):
    core = all_params["backend"]["core"]
    if core not in BACKENDS:
        raise NotImplementedError("The backend <" + core + "> has not yet been implemented")


def get_sim_config_and_inner_loop_step(all_params, stuff_for_time_loop, nt_in_loop, store_f_rules):
    """(sim_config, inner_loop) for a batch of nt_in_loop steps
    (vlapy/outer_loop.py:31-64)."""
    _check_backend(all_params)
    inner = get_inner_loop_stepper(all_params, stuff_for_time_loop, nt_in_loop)
    sim_config = get_arrays_for_inner_loop(stuff_for_time_loop, nt_in_loop, store_f_rules)
    return sim_config, inner


def get_everything_ready_for_outer_loop(diagnostics, all_params, pulse_dictionary, overall_num_steps):
    """Grids, initial f, time axis and driver (vlapy/outer_loop.py:67-146),
    without the MLflow logging of the reference."""
    f = initializers.initialize_distribution(nx=all_params["nx"], nv=all_params["nv"], vmax=all_params["vmax"])
    dx, x, kx, one_over_kx = initializers.initialize_spatial_quantities(
        xmin=all_params["xmin"], xmax=all_params["xmax"], nx=all_params["nx"])
    dv, v, kv = initializers.initialize_velocity_quantities(vmax=all_params["vmax"], nv=all_params["nv"])
    t_dummy = np.linspace(0, all_params["tmax"], all_params["nt"])
    dt = t_dummy[1] - t_dummy[0]
    t = dt * np.arange(overall_num_steps)
    driver_function = field_driver.get_driver_function(x=x, pulse_dictionary=pulse_dictionary)
    driver_array = field_driver.make_driver_array(function=driver_function, x_axis=x, time_axis=t)
    return {
        "e": np.zeros(x.size), "f": f, "nx": all_params["nx"], "kx": kx, "x": x,
        "one_over_kx": one_over_kx, "v": v, "kv": kv, "nv": all_params["nv"], "dv": dv,
        "driver": driver_array, "driver_function": driver_function, "dt": dt,
        "nu": all_params["nu"], "t": t, "rules_to_store_f": diagnostics.rules_to_store_f,
        "vlasov-poisson": all_params["vlasov-poisson"], "fokker-planck": all_params["fokker-planck"],
    }


def get_arrays_for_inner_loop(stuff_for_time_loop, nt_in_loop, store_f_rules, this_np=None, device=None):
    """sim_config dict of CUDA tensors (vlapy/outer_loop.py:149-215).  device
    defaults to the current CUDA device; "cpu" builds the same layout in host
    memory (for inspecting the layout without a GPU; the steps need CUDA)."""
    dev = torch.device(device) if device is not None else torch.device("cuda")
    if dev.type == "cuda":
        require_cuda()
    f0 = np.asarray(stuff_for_time_loop["f"], dtype=np.float64)
    e0 = np.asarray(stuff_for_time_loop["e"], dtype=np.float64)
    nx, nv = f0.shape
    put = (lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)) if dev.type != "cuda" else as_device
    if store_f_rules["space"] == "all":
        store_f = torch.zeros((nt_in_loop, nx, nv), dtype=torch.float64, device=dev)
        store_f[0] = put(f0)
    elif isinstance(store_f_rules["space"], list) and store_f_rules["space"][0] == "k0":
        m = len(store_f_rules["space"])
        first = np.fft.fft(f0, axis=0)[:m].astype(np.complex64)
        store_f = torch.zeros((nt_in_loop, m, nv), dtype=torch.complex64, device=dev)
        store_f[0] = torch.as_tensor(first, device=dev)
    else:
        raise NotImplementedError
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device=dev)  # noqa: E731
    return {
        "time_batch": z(nt_in_loop),
        "e": put(e0).clone(),
        "f": put(f0).clone(),
        "stored_f": store_f,
        "mean_cum_de2_previous": 0.0,
        "series": {k: z(nt_in_loop) for k in
                   ("mean_n", "mean_j", "mean_T", "mean_e2", "mean_de2", "mean_f2", "mean_flogf")},
        "fields": {k: z(nt_in_loop, nx) for k in ("e", "driver", "n", "j", "T", "q", "fv4", "vN")},
    }


def post_inner_loop_update(temp_storage, this_np=None):
    """Cumulative driver energy and the energy-balance series
    (vlapy/outer_loop.py:218-245), on the device."""
    se = temp_storage["series"]
    se["mean_cum_de2"] = temp_storage["mean_cum_de2_previous"] + torch.cumsum(se["mean_de2"], 0)
    se["mean_t_plus_e2_minus_cum_de2"] = se["mean_T"] + (se["mean_e2"] - se["mean_cum_de2"])
    se["mean_t_plus_e2_plus_cum_de2"] = se["mean_T"] + se["mean_e2"] + se["mean_de2"]
    temp_storage["mean_cum_de2_previous"] = float(se["mean_cum_de2"][-1])
    return temp_storage


def get_inner_loop_stepper(all_params, stuff_for_time_loop, steps_in_loop):
    """inner_loop(time_array, driver_array, temp_storage) running
    steps_in_loop steps (vlapy/outer_loop.py:248-281)."""
    _check_backend(all_params)
    one_step = step.get_timestep(all_params=all_params, stuff_for_time_loop=stuff_for_time_loop)
    drv = stuff_for_time_loop.get("driver_function")
    fused = hasattr(one_step, "plan") and (drv is None or isinstance(drv, PulseDriver))
    n_modes = step.n_modes_of(stuff_for_time_loop["rules_to_store_f"])
    plan = one_step.plan if fused else None
    side = torch.cuda.Stream() if fused else None

    def inner_loop(time_array, driver_array, temp_storage):
        tb = temp_storage.get("time_batch")
        db = temp_storage.get("driver_array_batch")
        ta = torch.as_tensor(np.asarray(time_array, dtype=np.float64))
        da = torch.as_tensor(np.asarray(driver_array, dtype=np.float64))
        # refill the batch buffers in place so a captured graph stays valid
        if isinstance(tb, torch.Tensor) and tb.is_cuda and tb.shape == ta.shape:
            tb.copy_(ta)
        else:
            temp_storage["time_batch"] = ta.cuda()
        if isinstance(db, torch.Tensor) and db.is_cuda and db.shape == da.shape:
            db.copy_(da)
        else:
            temp_storage["driver_array_batch"] = da.cuda()
        if fused:
            hist = history_struct(temp_storage, plan.nx, n_modes)
            state = temp_storage["f"]
            if plan.precision == "fp32-deltaf":
                # FP32 deviation from the run's fixed background, kept across
                # batches while the caller leaves f alone
                state = resident_deviation(plan, temp_storage)
            cur = torch.cuda.current_stream()
            side.wait_stream(cur)
            with torch.cuda.stream(side):
                plan.run_steps(state, temp_storage["e"], hist, temp_storage["time_batch"],
                               temp_storage["driver_array_batch"], 0, steps_in_loop, use_graph=True,
                               stream=side)
            cur.wait_stream(side)
            if plan.precision == "fp32-deltaf":
                publish_deviation(plan, temp_storage, state)
        else:
            for it in range(steps_in_loop):
                temp_storage, _ = one_step(temp_storage, it)
        post_inner_loop_update(temp_storage)
        return temp_storage

    inner_loop.plan = plan
    return inner_loop


__all__ = ["get_sim_config_and_inner_loop_step", "get_arrays_for_inner_loop", "get_inner_loop_stepper",
           "post_inner_loop_update", "get_everything_ready_for_outer_loop", "plan_for"]

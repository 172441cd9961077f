"""Host side of the reference's batched storage (vlapy/storage.py:56-67 and
:177-315).

``StorageManager.batch_update`` hands the arrays of a sim_config to xarray:
the series with coordinate (time), the fields with (time, space), stored_f
with (time, fourier_mode) or (time, space) and (velocity), and the current f
as one (time, space, velocity) record.  With this backend those arrays are
CUDA tensors, so they are brought to host memory first; the keys, shapes and
dtypes stay the reference's.  ``get_batched_data_from_sim_config`` is the
reference's helper of the same name with that copy added, and
``batch_coords`` lists the coordinates ``batch_update`` attaches, so a
caller (or a test without xarray) can check that every array fits them.
"""

from __future__ import annotations

import numpy as np


def to_host(a):
    """A NumPy array of a (CUDA or CPU) tensor, or a itself when it is not one."""
    if hasattr(a, "detach") and hasattr(a, "cpu"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def get_batched_data_from_sim_config(sim_config):
    """(fields, stored_f, time_batch, series, current_f) of a sim_config, as
    host NumPy arrays (vlapy/storage.py:56-67)."""
    fields = {k: to_host(v) for k, v in sim_config["fields"].items()}
    series = {k: to_host(v) for k, v in sim_config["series"].items()}
    return (fields, to_host(sim_config["stored_f"]), to_host(sim_config["time_batch"]), series,
            to_host(sim_config["f"]))


def batch_coords(time_actually_stored, xax, vax, rules_to_store_f):
    """The coordinates batch_update gives each kind of array
    (vlapy/storage.py:208-294): a dict kind -> list of (name, values)."""
    if not isinstance(rules_to_store_f, dict):
        raise NotImplementedError
    if rules_to_store_f["space"] == "all":
        second = ("space", np.asarray(xax))
    elif rules_to_store_f["space"][0] == "k0":
        m = len(rules_to_store_f["space"])
        second = ("fourier_mode", np.linspace(0, m - 1, m))
    else:
        raise NotImplementedError
    t = np.asarray(time_actually_stored)
    return {
        "full_distribution": [("time", t[-1:]), ("space", np.asarray(xax)), ("velocity", np.asarray(vax))],
        "series": [("time", t)],
        "fields": [("time", t), ("space", np.asarray(xax))],
        "distribution_function": [("time", t), second, ("velocity", np.asarray(vax))],
    }


def check_batch(sim_config, xax, vax, rules_to_store_f):
    """Bring a sim_config to the host and check every array against the
    coordinates batch_update attaches (what xarray.DataArray requires: one
    coordinate per axis, each as long as its axis).  Returns the host arrays
    in the layout of get_batched_data_from_sim_config."""
    fields, stored_f, t, series, f = get_batched_data_from_sim_config(sim_config)
    coords = batch_coords(t, xax, vax, rules_to_store_f)

    def fits(arr, cs, what):
        if arr.ndim != len(cs):
            raise ValueError("%s: %d axes for %d coordinates" % (what, arr.ndim, len(cs)))
        for ax, (name, vals) in enumerate(cs):
            if arr.shape[ax] != len(vals):
                raise ValueError("%s: axis %d (%s) has %d entries, coordinate %d"
                                 % (what, ax, name, arr.shape[ax], len(vals)))

    fits(np.expand_dims(f, axis=0), coords["full_distribution"], "full_distribution")
    for k, v in series.items():
        fits(v, coords["series"], "series " + k)
    for k, v in fields.items():
        fits(v, coords["fields"], "fields " + k)
    fits(stored_f, coords["distribution_function"], "distribution_function")
    return fields, stored_f, t, series, f

"""External field driver (vlapy/field_driver.py).

``get_driver_function`` returns a ``PulseDriver``: called with a time it
returns the driver on the host grid exactly as the reference closure does
(NumPy, so make_driver_array and the stored ``driver`` field match the
reference bit for bit), and it carries its pulse list so the time-step
kernels evaluate the same formula on the device at every sub-step time.
"""

from __future__ import annotations

import math

import numpy as np

from . import _lib


class PulseDriver:
    """Sum of pulses; envelope "tanh" is the reference's
    0.5*(tanh((t-tL)/twL) - tanh((t-tR)/twR)) * k * a0 * sin(k x - w t)
    (vlapy/field_driver.py:36-46); envelope "sin2" is
    a0 * sin^2(pi t / t_R) * sin(k x - w t) on [0, t_R] and zero after."""

    def __init__(self, x, pulse_dictionary):
        self.x = np.asarray(x, dtype=np.float64)
        self.pulse_dictionary = pulse_dictionary
        self.pulses = []
        for p in pulse_dictionary.values():
            env = p.get("envelope", "tanh")
            self.pulses.append({
                "k0": float(p["k0"]), "w0": float(p["w0"]), "a0": float(p["a0"]),
                "t_L": float(p.get("t_L", 0.0)), "t_R": float(p["t_R"]),
                "t_wL": float(p.get("t_wL", 1.0)), "t_wR": float(p.get("t_wR", 1.0)),
                "envelope": _lib.VG_ENV_SIN2 if env == "sin2" else _lib.VG_ENV_TANH,
            })

    def __call__(self, current_time):
        total = np.zeros(self.x.size)
        for p in self.pulses:
            kk, ww = p["k0"], p["w0"]
            if p["envelope"] == _lib.VG_ENV_SIN2:
                if current_time < 0.0 or current_time > p["t_R"]:
                    continue
                s = math.sin(math.pi * current_time / p["t_R"])
                total += (p["a0"] * (s * s)) * np.sin(kk * self.x - ww * current_time)
            else:
                envelope = 0.5 * (np.tanh((current_time - p["t_L"]) / p["t_wL"])
                                  - np.tanh((current_time - p["t_R"]) / p["t_wR"]))
                total += envelope * kk * p["a0"] * np.sin(kk * self.x - ww * current_time)
        return total


class ZeroDriver(PulseDriver):
    """No external field."""

    def __init__(self, x):
        super().__init__(x, {})


def get_driver_function(x, pulse_dictionary, np=None):  # noqa: A002 - reference signature
    """vlapy/field_driver.py:24-50.  The ``np`` argument is accepted for
    signature compatibility and ignored."""
    return PulseDriver(x, pulse_dictionary)


def make_driver_array(function, x_axis, time_axis):
    """Driver at every time of the run (vlapy/field_driver.py:53-62)."""
    out = np.zeros(time_axis.shape + x_axis.shape)
    for i in range(time_axis.size):
        out[i] = function(time_axis[i])
    return out


def get_driver_array_using_function(x, t, pulse_dictionary, this_np=None):
    """vlapy/field_driver.py:65-76."""
    return make_driver_array(get_driver_function(x, pulse_dictionary), x, t)

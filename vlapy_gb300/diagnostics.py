"""Post-run diagnostics of the field history (host side, NumPy).

The reference estimates the damping rate of an electron plasma wave by
averaging d log|E_k|/dt over a window (vlapy/diagnostics/low_level_helpers.py:
69-87), which is biased for an undriven, standing wave: |E_k| of a standing
wave oscillates between peaks and zeros.  Here the rate is the slope of a
least-squares line through the logarithm of the peak heights of |E_k|(t),
each peak refined by a parabola through its three samples in log space, and
the frequency follows from the mean peak spacing (|E_k| of a standing wave
peaks twice per period).
"""

from __future__ import annotations

import numpy as np


def mode_amplitude(e_hist, mode=1):
    """|FFT_x(E)[mode]| of a field history [steps][nx]."""
    return np.abs(np.fft.fft(np.asarray(e_hist), axis=1)[:, mode])


def damping_fit(t, amp, t_min=None, t_max=None):
    """(rate, frequency) from the peaks of amp(t) in [t_min, t_max]; NaNs when
    the window holds fewer than three peaks."""
    t = np.asarray(t, dtype=np.float64)
    amp = np.asarray(amp, dtype=np.float64)
    keep = np.ones(t.shape, dtype=bool)
    if t_min is not None:
        keep &= t >= t_min
    if t_max is not None:
        keep &= t <= t_max
    ts, a = t[keep], amp[keep]
    if a.size < 3:
        return float("nan"), float("nan")
    mid = a[1:-1]
    peaks = np.flatnonzero((mid > a[:-2]) & (mid >= a[2:])) + 1
    if peaks.size < 3 or np.any(a[peaks - 1] <= 0) or np.any(a[peaks + 1] <= 0):
        return float("nan"), float("nan")
    la, lb, lc = np.log(a[peaks - 1]), np.log(a[peaks]), np.log(a[peaks + 1])
    curv = la - 2.0 * lb + lc
    shift = np.where(curv != 0.0, 0.5 * (la - lc) / np.where(curv != 0.0, curv, 1.0), 0.0)
    dt = ts[1] - ts[0]
    t_peak = ts[peaks] + shift * dt
    log_peak = lb - 0.25 * (la - lc) * shift
    rate = np.polyfit(t_peak, log_peak, 1)[0]
    freq = np.pi / np.mean(np.diff(t_peak))
    return float(rate), float(freq)

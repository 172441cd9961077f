"""Batched parameter sweep: thousands of independent VlaPy runs on one GPU.

Each run is the reference's leapfrog step (exponential advection in x and v,
spectral Poisson, the Dougherty or Lenard-Bernstein collision step for nu > 0;
vlapy/core/step.py:286-328) from f = M(v) (1 + A cos(k x)) on x in [0, 2 pi/k),
v in [-vmax, vmax), in the FP32 delta-f arithmetic of the GB300 step.  The
reference runs one simulation per process; here every kernel launch of a step
covers all runs (libvlagpu vg_sweep_*), and a whole batch of steps replays as
one CUDA graph.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check
from .plan import _prof_dict, ptr, require_cuda, stream_handle

SERIES = ("mean_n", "mean_j", "mean_T", "mean_e2", "mean_de2", "mean_f2", "mean_flogf")


def sweep_config(n_runs=4096, seed=20261203, nx_choices=(32, 64, 128), nv_choices=(256, 512, 1024),
                 k_range=(0.25, 0.45), log_amp=(-6.0, -2.0), log_nu=(-5.0, -2.0), p_collisionless=0.25):
    """Seeded run list of the batched-sweep workload: nx and nv uniform over
    the choices, k ~ U[0.25, 0.45], amplitude and nu log-uniform, a quarter of
    the runs collisionless."""
    rng = np.random.default_rng(seed)
    nx = rng.choice(np.asarray(nx_choices), n_runs)
    nv = rng.choice(np.asarray(nv_choices), n_runs)
    k = rng.uniform(k_range[0], k_range[1], n_runs)
    amp = 10.0 ** rng.uniform(log_amp[0], log_amp[1], n_runs)
    nu = 10.0 ** rng.uniform(log_nu[0], log_nu[1], n_runs)
    nu[rng.random(n_runs) < p_collisionless] = 0.0
    return [dict(nx=int(a), nv=int(b), k=float(c), amplitude=float(d), nu=float(e))
            for a, b, c, d, e in zip(nx, nv, k, amp, nu)]


class _DeviceArray:
    """__cuda_array_interface__ of a device buffer owned by the library; it
    holds its owner, and a tensor made from it holds this object."""

    def __init__(self, owner, ptr_value, shape, typestr):
        self.owner = owner
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr_value), False),
                                         "version": 2, "strides": None}


class Sweep:
    """Owns a vg_sweep; runs are advanced together on the current stream."""

    def __init__(self, runs, vmax=6.4, dt=0.1, collision="dg"):
        require_cuda()
        self._lib = _lib.load()
        self.runs = list(runs)
        self.vmax, self.dt = float(vmax), float(dt)
        arr = (_lib.VgSweepRun * len(self.runs))()
        for i, r in enumerate(self.runs):
            arr[i] = _lib.VgSweepRun(int(r["nx"]), int(r["nv"]), float(r["k"]), float(r["amplitude"]),
                                     float(r["nu"]))
        d = _lib.VgSweepDesc(len(self.runs), _lib.VG_COLL_DG if collision == "dg" else _lib.VG_COLL_LB,
                             self.vmax, self.dt, arr)
        h = C.c_void_p()
        check(self._lib.vg_sweep_create(C.byref(d), C.byref(h)), "sweep create")
        self._h = h
        cells, xp = C.c_int64(), C.c_int64()
        check(self._lib.vg_sweep_sizes(h, C.byref(cells), C.byref(xp)), "sweep sizes")
        self.cells, self.x_points = int(cells.value), int(xp.value)
        offs = (C.c_int64 * len(self.runs))()
        check(self._lib.vg_sweep_x_offsets(h, offs), "sweep offsets")
        self.x_offsets = np.array(offs[:], dtype=np.int64)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.vg_sweep_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_runs(self):
        return len(self.runs)

    def reset(self, stream=None):
        check(self._lib.vg_sweep_reset(self._h, stream_handle(stream)), "sweep reset")

    def history(self, rows):
        """Device buffers for `rows` stored steps: e [rows][x_points] and
        series [rows][n_runs][7]."""
        dev = torch.device("cuda")
        return (torch.zeros((rows, self.x_points), dtype=torch.float64, device=dev),
                torch.zeros((rows, self.n_runs, 7), dtype=torch.float64, device=dev))

    def run_steps(self, nsteps, e_hist=None, series_hist=None, row0=0, use_graph=False, stream=None):
        rows = 0
        if e_hist is not None:
            rows = int(e_hist.shape[0])
        elif series_hist is not None:
            rows = int(series_hist.shape[0])
        check(self._lib.vg_sweep_run_steps(self._h, int(nsteps), ptr(e_hist), ptr(series_hist), rows, int(row0),
                                           int(bool(use_graph)), stream_handle(stream)), "sweep run steps")

    def read_run(self, i, stream=None):
        """(f [nx][nv] float64, e [nx] float64) of run i on the device."""
        r = self.runs[i]
        f = torch.empty((r["nx"], r["nv"]), dtype=torch.float64, device="cuda")
        e = torch.empty(r["nx"], dtype=torch.float64, device="cuda")
        check(self._lib.vg_sweep_read_run(self._h, int(i), ptr(f), ptr(e), stream_handle(stream)), "sweep read")
        return f, e

    @property
    def g_offsets(self):
        """Start of each run's [nx][nv] block in the packed state (runs back to back)."""
        sizes = np.array([r["nx"] * r["nv"] for r in self.runs], dtype=np.int64)
        return np.concatenate([[0], np.cumsum(sizes)[:-1]])

    def _state_buffer(self, t, n, dtype, what):
        if t is None:
            return None
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()
                and t.numel() == n):
            raise ValueError(f"{what} must be a contiguous CUDA {dtype} tensor of {n} elements")
        return t

    def get_state(self, g_out=None, e_out=None, stream=None):
        """Packed FP32 deviations g [cells] and fields e [x_points] of all runs."""
        if g_out is None:
            g_out = torch.empty(self.cells, dtype=torch.float32, device="cuda")
        if e_out is None:
            e_out = torch.empty(self.x_points, dtype=torch.float64, device="cuda")
        self._state_buffer(g_out, self.cells, torch.float32, "g_out")
        self._state_buffer(e_out, self.x_points, torch.float64, "e_out")
        check(self._lib.vg_sweep_get_state(self._h, ptr(g_out), ptr(e_out), stream_handle(stream)), "sweep get")
        return g_out, e_out

    def set_state(self, g_in=None, e_in=None, stream=None):
        """Overwrite g and/or e of all runs (layouts as get_state)."""
        g_in = self._state_buffer(g_in, self.cells, torch.float32, "g_in")
        e_in = self._state_buffer(e_in, self.x_points, torch.float64, "e_in")
        check(self._lib.vg_sweep_set_state(self._h, ptr(g_in), ptr(e_in), stream_handle(stream)), "sweep set")

    def state_view(self):
        """The sweep's own FP32 state g [cells] as a CUDA tensor (no copy; the
        tensor keeps the sweep alive; g may be modified between run_steps
        calls on the same stream)."""
        gp = C.c_void_p()
        check(self._lib.vg_sweep_state_ptr(self._h, C.byref(gp), None), "sweep state")
        return torch.as_tensor(_DeviceArray(self, gp.value, (self.cells,), "<f4"), device="cuda")

    def damping(self, e_hist, t0=None, t_min=5.0, t_max=None, stream=None):
        """(rate, frequency) float64 CUDA tensors [n_runs] of every run, fitted
        on the device to the peaks of |E_1|(t) of an e history whose row k is
        time t0 + k dt (t0 defaults to dt: the history of run_steps from a
        reset); NaN for a run with fewer than three peaks in the window."""
        rows = int(e_hist.shape[0])
        if not (isinstance(e_hist, torch.Tensor) and e_hist.is_cuda and e_hist.dtype == torch.float64
                and e_hist.is_contiguous() and tuple(e_hist.shape) == (rows, self.x_points)):
            raise ValueError("e_hist must be a contiguous CUDA float64 tensor [rows][x_points]")
        t0 = self.dt if t0 is None else float(t0)
        t_max = t0 + (rows - 1) * self.dt if t_max is None else float(t_max)
        rate = torch.empty(self.n_runs, dtype=torch.float64, device="cuda")
        freq = torch.empty(self.n_runs, dtype=torch.float64, device="cuda")
        check(self._lib.vg_sweep_damping(self._h, ptr(e_hist), rows, t0, float(t_min), t_max, ptr(rate), ptr(freq),
                                         stream_handle(stream)), "sweep damping")
        return rate, freq

    def e_of(self, e_hist, i):
        """e history [rows][nx] of run i from a sweep e-history buffer."""
        o = int(self.x_offsets[i])
        return e_hist[:, o:o + self.runs[i]["nx"]]

    def status(self):
        """(flags, uses_tma) after synchronising the device: the status bits
        since creation (a VlagpuError with VG_ERR_TIMEOUT when a bounded wait
        of the TMA x-drift ran out, else with VG_ERR_NUMERIC when a field solve
        produced NaN or Inf) and whether the x-drift loads its tiles through
        the TMA."""
        flags, tma = C.c_int32(), C.c_int32()
        check(self._lib.vg_sweep_status(self._h, C.byref(flags), C.byref(tma)), "sweep status")
        return int(flags.value), bool(tma.value)

    def set_wait_limit(self, ns):
        """Limit, in ns, of the TMA x-drift's waits for its tiles (default
        2e9).  A wait that runs out marks the sweep's status and ends its CTA."""
        check(self._lib.vg_sweep_set_wait_limit(self._h, int(ns)), "sweep wait limit")

    def inject_lost_tiles(self, on=True):
        """Test hook: while on, the TMA x-drift requests no tiles, so each of
        its waits runs out after the wait limit (the steps are not valid; the
        status reports the timeout)."""
        check(self._lib.vg_sweep_inject_lost_tiles(self._h, int(bool(on))), "sweep inject")

    def set_step_events(self, events):
        """torch.cuda.Event objects that each following run_steps call records
        after step k has stored its history row (k < len(events)), so that
        another stream can copy that row out while the later steps run; an
        empty list clears them.  The events are recorded once here on the
        current stream (which creates them) and must outlive their use."""
        events = list(events)
        for ev in events:
            ev.record()
        handles = (C.c_void_p * max(1, len(events)))(*[C.c_void_p(ev.cuda_event) for ev in events])
        if any(h is None or h == 0 for h in (ev.cuda_event for ev in events)):
            raise ValueError("every step event must be a created CUDA event")
        check(self._lib.vg_sweep_set_step_events(self._h, handles, len(events)), "sweep step events")
        self._step_events = events  # keep them alive while they are set

    def profile(self, enable):
        check(self._lib.vg_sweep_profile_enable(self._h, int(bool(enable))), "profile")

    def profile_read(self):
        buf = (_lib.VgProfEntry * 16)()
        n = C.c_int32()
        check(self._lib.vg_sweep_profile_read(self._h, buf, 16, C.byref(n)), "profile read")
        return _prof_dict(buf, n.value)

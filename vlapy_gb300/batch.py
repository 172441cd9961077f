"""Batched FP64 step: many independent runs of the reference's FP64 time step
on one GPU (libvlagpu vg_batch_*).

Each run is the reference's leapfrog step with exponential advection, the
spectral Poisson solve, the implicit collision step (Dougherty or
Lenard-Bernstein, skipped for nu = 0) and the per-step moments
(vlapy/core/step.py:286-328), on the reference's grids (vlapy/initializers.py:
56-89, computed here with NumPy as the reference computes them).  Every run
goes through the same device code as a single vg_plan, so the batch follows
the reference's NumPy step as a plan does (<= 1e-12 per step), while every
kernel launch covers all runs of one shape.  This is the plain FP64 GPU
method the FP32 delta-f sweep (vlapy_gb300.sweep) is measured against.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib, initializers
from ._lib import check
from .plan import _prof_dict, ptr, require_cuda, stream_handle


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class Batch64:
    """Owns a vg_batch over runs given as the sweep's dicts {nx, nv, k,
    amplitude, nu} (x in [0, 2 pi / k), v in [-vmax, vmax)).  The runs are
    stored grouped by nv (the batch's layout); ``order[i]`` is the input index
    of stored run i and every public method takes and returns input indices."""

    def __init__(self, runs, vmax=6.4, dt=0.1, collision="dg"):
        require_cuda()
        self._lib = _lib.load()
        self.runs = [dict(r) for r in runs]
        self.vmax, self.dt = float(vmax), float(dt)
        if collision not in ("dg", "lb"):
            raise NotImplementedError("Collision Operator: <%s> has not yet been implemented" % collision)
        self.order = np.array(sorted(range(len(self.runs)), key=lambda i: (self.runs[i]["nv"], i)), dtype=np.int64)
        self.slot = np.empty_like(self.order)
        self.slot[self.order] = np.arange(len(self.order))
        descs = (_lib.VgRunDesc * len(self.runs))()
        self._keep = []
        vgrid = {}
        for j, i in enumerate(self.order):
            r = self.runs[i]
            nx, nv, k = int(r["nx"]), int(r["nv"]), float(r["k"])
            dx, x, kx, inv = initializers.initialize_spatial_quantities(0.0, 2.0 * np.pi / k, nx)
            if nv not in vgrid:
                dv, v, kv = initializers.initialize_velocity_quantities(self.vmax, nv)
                v = _f64(v)
                vpow = _f64(np.stack([v ** 2.0, v ** 2, v ** 3, v ** 4, v ** 5]))
                vgrid[nv] = (float(dv), v, _f64(kv), vpow)
            dv, v, kv, vpow = vgrid[nv]
            arrs = (_f64(x), _f64(kx), _f64(inv))
            self._keep.append(arrs)
            d = descs[j]
            d.nx, d.nv = nx, nv
            d.precision = _lib.VG_F64
            nu = float(r["nu"])
            d.collision = (_lib.VG_COLL_DG if collision == "dg" else _lib.VG_COLL_LB) if nu > 0 else _lib.VG_COLL_NONE
            d.integrator = _lib.VG_LEAPFROG
            d.n_pulses = 0
            d.dt, d.nu, d.dx, d.dv = self.dt, nu, float(dx), dv
            d.dv_sq = dv ** 2.0
            d.x, d.kx, d.one_over_kx = (a.ctypes.data_as(_lib.DP) for a in arrs)
            d.v, d.kv, d.v_pow = v.ctypes.data_as(_lib.DP), kv.ctypes.data_as(_lib.DP), vpow.ctypes.data_as(_lib.DP)
            d.pulses = None
            d.f_background = None
        self._vgrid = vgrid
        h = C.c_void_p()
        check(self._lib.vg_batch_create(descs, len(self.runs), C.byref(h)), "batch create")
        self._h = h
        cells, xp = C.c_int64(), C.c_int64()
        check(self._lib.vg_batch_sizes(h, C.byref(cells), C.byref(xp)), "batch sizes")
        self.cells, self.x_points = int(cells.value), int(xp.value)
        sizes = np.array([self.runs[i]["nx"] * self.runs[i]["nv"] for i in self.order], dtype=np.int64)
        xs = np.array([self.runs[i]["nx"] for i in self.order], dtype=np.int64)
        # offsets of the stored runs, indexed by input run
        self.f_offsets = np.empty(len(self.runs), dtype=np.int64)
        self.x_offsets = np.empty(len(self.runs), dtype=np.int64)
        self.f_offsets[self.order] = np.concatenate([[0], np.cumsum(sizes)[:-1]])
        self.x_offsets[self.order] = np.concatenate([[0], np.cumsum(xs)[:-1]])

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.vg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_runs(self):
        return len(self.runs)

    def initial_state(self):
        """(f [cells], e [x_points]) float64 CUDA tensors: every run's
        f = M(v) (1 + A cos(k x)) with M the trapz-normalised Maxwellian of
        vlapy/initializers.py:29-53, formed elementwise in FP64 on the device
        (the same products NumPy forms), and e = 0."""
        dev = torch.device("cuda")
        f = torch.empty(self.cells, dtype=torch.float64, device=dev)
        maxw = {nv: torch.as_tensor(_f64(initializers.initialize_distribution(1, nv, self.vmax)[0]), device=dev)
                for nv in self._vgrid}
        for i, r in enumerate(self.runs):
            nx, nv = int(r["nx"]), int(r["nv"])
            dx, x, kx, inv = initializers.initialize_spatial_quantities(0.0, 2.0 * np.pi / float(r["k"]), nx)
            pert = torch.as_tensor(_f64(1.0 + float(r["amplitude"]) * np.cos(float(r["k"]) * x)), device=dev)
            o = int(self.f_offsets[i])
            f[o:o + nx * nv].view(nx, nv).copy_(maxw[nv][None, :] * pert[:, None])
        return f, torch.zeros(self.x_points, dtype=torch.float64, device=dev)

    def history(self, rows):
        """Device buffers for `rows` stored steps: e [rows][x_points] (runs at
        x_offsets) and series [rows][n_runs][7] (rows in stored order: use
        series_of)."""
        dev = torch.device("cuda")
        return (torch.zeros((rows, self.x_points), dtype=torch.float64, device=dev),
                torch.zeros((rows, self.n_runs, 7), dtype=torch.float64, device=dev))

    def run_steps(self, f, e, nsteps, e_hist=None, series_hist=None, row0=0, use_graph=False, stream=None):
        for t, n, what in ((f, self.cells, "f"), (e, self.x_points, "e")):
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()
                    and t.numel() == n):
                raise ValueError("%s must be a contiguous CUDA float64 tensor of %d elements" % (what, n))
        rows = 0
        if e_hist is not None:
            rows = int(e_hist.shape[0])
        elif series_hist is not None:
            rows = int(series_hist.shape[0])
        check(self._lib.vg_batch_run_steps(self._h, ptr(f), ptr(e), int(nsteps), ptr(e_hist), ptr(series_hist),
                                           rows, int(row0), int(bool(use_graph)), stream_handle(stream)),
              "batch run steps")

    def f_of(self, f, i):
        """f [nx][nv] of input run i (a view of the packed state)."""
        r = self.runs[i]
        o = int(self.f_offsets[i])
        return f[o:o + r["nx"] * r["nv"]].view(r["nx"], r["nv"])

    def e_of(self, e, i):
        """e [..., nx] of input run i from a packed e or an e history."""
        o = int(self.x_offsets[i])
        return e[..., o:o + self.runs[i]["nx"]]

    def series_of(self, series_hist, i):
        """series [rows][7] of input run i."""
        return series_hist[:, int(self.slot[i])]

    def status(self):
        """Status bits the batch's kernels raised since it was created
        (synchronises the device); a VlagpuError with VG_ERR_NUMERIC when a
        field solve produced NaN or Inf."""
        flags = C.c_int32()
        check(self._lib.vg_batch_status(self._h, C.byref(flags)), "batch status")
        return int(flags.value)

    def profile(self, enable):
        check(self._lib.vg_batch_profile_enable(self._h, int(bool(enable))), "profile")

    def profile_read(self):
        buf = (_lib.VgProfEntry * 16)()
        n = C.c_int32()
        check(self._lib.vg_batch_profile_read(self._h, buf, 16, C.byref(n)), "profile read")
        return _prof_dict(buf, n.value)

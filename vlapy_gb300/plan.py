"""Host-side plan object: builds a vg_plan from the reference's derived
quantities (stuff_for_time_loop, vlapy/outer_loop.py:125-144) and owns it.

Grids are computed on the host with NumPy exactly as the reference does
(vlapy/initializers.py:56-89) and copied once to the device, so the kernels
see bit-identical axes, wavenumbers and velocity powers.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check

COLLISIONS = {"none": _lib.VG_COLL_NONE, "lb": _lib.VG_COLL_LB, "dg": _lib.VG_COLL_DG}
INTEGRATORS = {"leapfrog": _lib.VG_LEAPFROG, "pefrl": _lib.VG_PEFRL, "h-sixth": _lib.VG_H_SIXTH}
PRECISIONS = {"fp64": _lib.VG_F64, "fp32-deltaf": _lib.VG_F32_DELTA_F}


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_lib.DP)


def stream_handle(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def ptr(t) -> int:
    """Device pointer of a CUDA tensor (or 0 for None); refuses host tensors."""
    if t is None:
        return 0
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("expected a CUDA tensor, got %r" % (type(t),))
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return int(t.data_ptr())


def check_f64(t, shape, name):
    """Refuse a tensor that is not float64 of the given shape before its pointer
    reaches a kernel (the out-of-place steppers index nx * nv cells of it)."""
    if not isinstance(t, torch.Tensor):
        raise TypeError("%s: expected a tensor, got %r" % (name, type(t)))
    if t.dtype != torch.float64 or tuple(t.shape) != tuple(shape):
        raise ValueError("%s: expected float64 of shape %s, got %s of shape %s"
                         % (name, tuple(shape), t.dtype, tuple(t.shape)))
    return t


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("vlapy_gb300 needs a CUDA device (GB300); none is available")


class Plan:
    """Owns one vg_plan.  Not thread-safe; calls are ordered on a stream."""

    def __init__(self, nx, nv, x, v, kx, kv, one_over_kx, dx, dv, dt=0.0, nu=0.0,
                 collision="none", integrator="leapfrog", pulses=None,
                 precision="fp64", f_background=None):
        require_cuda()
        lib = _lib.load()
        if collision not in COLLISIONS:
            raise NotImplementedError("Collision Operator: <%s> has not yet been implemented" % collision)
        if integrator not in INTEGRATORS:
            raise NotImplementedError("df/dt : <%s> has not yet been implemented" % integrator)
        self.nx, self.nv = int(nx), int(nv)
        self.dt, self.nu, self.dv, self.dx = float(dt), float(nu), float(dv), float(dx)
        self.collision, self.integrator, self.precision = collision, integrator, precision
        f64 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64))  # noqa: E731
        self._x, self._v, self._kx = f64(x), f64(v), f64(kx)
        self._kv, self._inv = f64(kv), f64(one_over_kx)
        v_arr = self._v
        # the exact expressions the reference evaluates (vlapy/core/collisions.py:57,
        # vlapy/core/step.py:168-171)
        self._vpow = np.ascontiguousarray(np.stack(
            [v_arr ** 2.0, v_arr ** 2, v_arr ** 3, v_arr ** 4, v_arr ** 5]))
        pl = list(pulses or [])
        self._pulses = (_lib.VgPulse * max(1, len(pl)))()
        for i, p in enumerate(pl):
            self._pulses[i] = _lib.VgPulse(p["k0"], p["w0"], p["a0"], p["t_L"], p["t_R"],
                                           p.get("t_wL", 1.0), p.get("t_wR", 1.0),
                                           p.get("envelope", _lib.VG_ENV_TANH), 0)
        self._fbg = None if f_background is None else f64(f_background)
        d = _lib.VgRunDesc()
        d.nx, d.nv = self.nx, self.nv
        d.precision = PRECISIONS[precision]
        d.collision = COLLISIONS[collision]
        d.integrator = INTEGRATORS[integrator]
        d.n_pulses = len(pl)
        d.dt, d.nu, d.dx, d.dv = self.dt, self.nu, self.dx, self.dv
        d.dv_sq = self.dv ** 2.0
        d.x, d.v, d.kx, d.kv = _dp(self._x), _dp(self._v), _dp(self._kx), _dp(self._kv)
        d.one_over_kx = _dp(self._inv)
        d.v_pow = _dp(self._vpow)
        d.pulses = C.cast(self._pulses, C.POINTER(_lib.VgPulse))
        d.f_background = _dp(self._fbg) if self._fbg is not None else None
        self._desc = d
        h = C.c_void_p()
        check(lib.vg_plan_create(C.byref(d), C.byref(h)), "plan create")
        self._h = h
        self._lib = lib

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.vg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- sub-operators -------------------------------------------------
    def edfdv(self, f, e, dt, stream=None):
        check(self._lib.vg_edfdv(self._h, ptr(f), ptr(e), float(dt), stream_handle(stream)), "edfdv")
        return f

    def vdfdx(self, f, dt, stream=None):
        check(self._lib.vg_vdfdx(self._h, ptr(f), float(dt), stream_handle(stream)), "vdfdx")
        return f

    def _alt_args(self, name, f, out, e=None):
        if self.precision != "fp64":
            raise NotImplementedError(name + " is implemented in the fp64 precision mode only")
        grid = (self.nx, self.nv)
        check_f64(f, grid, name + " f")
        check_f64(out, grid, name + " out")
        if e is not None:
            check_f64(e, (self.nx,), name + " e")

    def vdfdx_sl(self, f, out, dt, stream=None):
        """Semi-Lagrangian x step of f into out (FP64 plans; out must not be f)."""
        self._alt_args("vdfdx sl", f, out)
        check(self._lib.vg_vdfdx_sl(self._h, ptr(f), ptr(out), float(dt), stream_handle(stream)), "vdfdx sl")
        return out

    def edfdv_sl(self, f, e, out, dt, stream=None):
        """Semi-Lagrangian v step of f into out (FP64 plans; out must not be f)."""
        self._alt_args("edfdv sl", f, out, e)
        check(self._lib.vg_edfdv_sl(self._h, ptr(f), ptr(e), ptr(out), float(dt), stream_handle(stream)),
              "edfdv sl")
        return out

    def edfdv_cd2(self, f, e, out, dt, stream=None):
        """Centred-difference v step of f into out (FP64 plans; out must not be f)."""
        self._alt_args("edfdv cd2", f, out, e)
        check(self._lib.vg_edfdv_cd2(self._h, ptr(f), ptr(e), ptr(out), float(dt), stream_handle(stream)),
              "edfdv cd2")
        return out

    def charge_density(self, f, out, stream=None):
        check(self._lib.vg_charge_density(self._h, ptr(f), ptr(out), stream_handle(stream)), "density")
        return out

    def poisson(self, rho, out, stream=None):
        check(self._lib.vg_poisson(self._h, ptr(rho), ptr(out), stream_handle(stream)), "poisson")
        return out

    def field_solve(self, f, driver, out, stream=None):
        check(self._lib.vg_field_solve(self._h, ptr(f), ptr(driver), ptr(out), stream_handle(stream)),
              "field solve")
        return out

    def collision_step(self, f, stream=None):
        check(self._lib.vg_collision_step(self._h, ptr(f), stream_handle(stream)), "collision step")
        return f

    def driver(self, t, out, stream=None):
        check(self._lib.vg_driver(self._h, float(t), ptr(out), stream_handle(stream)), "driver")
        return out

    def storage_step(self, f, e, de, hist, i, stream=None):
        check(self._lib.vg_storage_step(self._h, ptr(f), ptr(e), ptr(de), C.byref(hist), int(i),
                                        stream_handle(stream)), "storage step")

    def status(self):
        """Status bits the plan's kernels raised since it was created
        (synchronises the device); a VlagpuError with VG_ERR_NUMERIC when a
        field solve produced NaN or Inf."""
        flags = C.c_int32()
        check(self._lib.vg_plan_status(self._h, C.byref(flags)), "plan status")
        return int(flags.value)

    def profile(self, enable: bool):
        check(self._lib.vg_profile_enable(self._h, int(bool(enable))), "profile")

    def profile_read(self):
        """{kernel: {launches, total_ms, bytes_per_launch}} since the last read."""
        buf = (_lib.VgProfEntry * 16)()
        n = C.c_int32()
        check(self._lib.vg_profile_read(self._h, buf, 16, C.byref(n)), "profile read")
        return _prof_dict(buf, n.value)

    def run_steps(self, f, e, hist, time_batch, driver_batch, i0, nsteps, use_graph=False, stream=None):
        hp = C.byref(hist) if hist is not None else None
        check(self._lib.vg_run_steps(self._h, ptr(f), ptr(e), hp, ptr(time_batch), ptr(driver_batch),
                                     int(i0), int(nsteps), int(bool(use_graph)), stream_handle(stream)),
              "run steps")


def _prof_dict(entries, n):
    out = {}
    for i in range(n):
        e = entries[i]
        out[e.name.decode()] = {"launches": int(e.launches), "total_ms": float(e.total_ms),
                                "bytes_per_launch": float(e.bytes_per_launch)}
    return out


def history_struct(storage: dict, nx: int, n_modes: int | None):
    """vg_history over the torch tensors of a temp_storage dict
    (vlapy/outer_loop.py:190-215).  n_modes None means the store-all rule."""
    h = _lib.VgHistory()
    series_keys = ("mean_n", "mean_j", "mean_T", "mean_e2", "mean_de2", "mean_f2", "mean_flogf")
    field_keys = ("e", "driver", "n", "j", "T", "q", "fv4", "vN")
    stored = storage["stored_f"]
    h.nt = int(stored.shape[0])
    for i, k in enumerate(field_keys):
        h.fields[i] = ptr(storage["fields"][k])
    for i, k in enumerate(series_keys):
        h.series[i] = ptr(storage["series"][k])
    h.stored_f = ptr(stored)
    if n_modes is None:
        h.store_all, h.n_modes, h.n_slots = 1, 0, 0
    else:
        h.store_all = 0
        h.n_modes = int(n_modes)
        h.n_slots = int(stored.shape[1])
    return h

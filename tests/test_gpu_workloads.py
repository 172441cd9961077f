"""The FP32 delta-f step on the two single-run workloads, checked against the
FP64 GPU step.

* Driven electron plasma wave: 64 x 1024, k = 0.3, vmax = 6.4, Maxwellian
  start, Dougherty collisions nu = 1e-3, dt = 0.1, 4000 steps, external field
  a0 sin(k x - w t) sin^2(pi t / 100) on [0, 100] with a0 = 1e-2 and w the
  dispersion root.
* Large two-stream run: 4096 x 8192, x in [0, 2 pi / 0.3), vmax = 8,
  f = (M(v - 3) + M(v + 3)) / 2 (1 + 1e-3 sum_{m=1..16} cos(m k x + phi_m))
  with phi_m from default_rng(4), Dougherty nu = 1e-4, dt = 0.05.

The reference solution is the FP64 GPU step, which follows the reference's NumPy step to
<= 1e-12 per step (tests/test_gpu_parity.py, including the reference's own
steps of the driven workload's grid and driver in the fixture
driven_sin2_dg_64x1024).  It stands in for the CPU oracle here because the
oracle needs minutes (4000 steps of 64 x 1024) to hours (4096 x 8192) for
these runs.  Errors are relative L2: f against the size of its deviation
from the initial x-mean, e over the whole stored history, and the
field-energy history (mean e^2 per step).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import vlapy_oracle as vo  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_loaded():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import _lib
    _lib.load()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _run(precision, f, f_bg, grids, nsteps, dt, nu, pulses, n_store):
    """nsteps fused steps of one plan; returns (f, e, e history, mean e^2)."""
    from vlapy_gb300.plan import Plan, history_struct
    from vlapy_gb300 import field_driver
    x, v, kx, kv, inv, dx, dv = grids
    nx, nv = f.shape
    dev = torch.device("cuda")
    p = Plan(nx, nv, x, v, kx, kv, inv, dx, dv, dt=dt, nu=nu, collision="dg", pulses=pulses,
             precision=precision, f_background=f_bg if precision != "fp64" else None)
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device=dev)  # noqa: E731
    st = {"stored_f": torch.zeros((n_store, 1, nv), dtype=torch.complex64, device=dev),
          "fields": {k: z(n_store, nx) for k in vo.FIELD_KEYS},
          "series": {k: z(n_store) for k in vo.SERIES_KEYS}}
    if precision == "fp64":
        state = torch.as_tensor(f, device=dev)
    else:
        state = torch.as_tensor((f - f_bg[None, :]).astype(np.float32), device=dev)
    e = z(nx)
    tb = torch.as_tensor(dt * np.arange(nsteps), device=dev)
    if pulses:
        drv = field_driver.get_driver_function(x, {"p": dict(pulses[0], envelope="sin2")})
        db = torch.as_tensor(field_driver.make_driver_array(drv, x, dt * np.arange(nsteps)), device=dev)
    else:
        db = z(nsteps, nx)
    e_hist, e2 = [], []
    for i0 in range(0, nsteps, n_store):
        n = min(n_store, nsteps - i0)
        hist = history_struct(st, nx, 1)
        # the history arrays hold n_store rows: storage index i lands in row i - i0
        p.run_steps(state, e, hist, tb[i0:], db[i0:], 0, n, use_graph=False)
        e_hist.append(st["fields"]["e"][:n].cpu().numpy().copy())
        e2.append(st["series"]["mean_e2"][:n].cpu().numpy().copy())
    torch.cuda.synchronize()
    fo = state.cpu().numpy()
    if precision != "fp64":
        fo = fo.astype(np.float64) + f_bg[None, :]
    return fo, e.cpu().numpy(), np.concatenate(e_hist), np.concatenate(e2)


def test_driven_wave_fp32_against_fp64_4000_steps():
    """The driven-wave workload over its full 4000 steps (t = 0..400: the
    sin^2 drive to t = 100, then the free wave under collisions).  The gate:
    field-energy history within 1e-3 of the FP64 step.  The
    e and f errors grow in the driven, nonlinear phase; a second FP64 run
    started from f perturbed by 1e-7 (relative, seeded noise: FP32's rounding
    level) shows how much of that growth is the dynamics' own sensitivity."""
    from vlapy_gb300 import dispersion
    nx, nv, k, vmax, dt, nu, nsteps = 64, 1024, 0.3, 6.4, 0.1, 1e-3, 4000
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    dv, v, kv = vo.velocity_axis(vmax, nv)
    w = float(np.real(dispersion.get_roots_to_electrostatic_dispersion(1.0, 1.0, k)))
    pulses = [{"k0": k, "w0": w, "a0": 1e-2, "t_L": 0.0, "t_R": 100.0, "envelope": 1}]
    f = vo.maxwellian(nx, nv, vmax)
    fbg = f.mean(axis=0)
    grids = (x, v, kx, kv, inv, dx, dv)
    f64, e64, eh64, w64 = _run("fp64", f, fbg, grids, nsteps, dt, nu, pulses, 1000)
    f32, e32, eh32, w32 = _run("fp32-deltaf", f, fbg, grids, nsteps, dt, nu, pulses, 1000)
    fp = f * (1.0 + 1e-7 * np.random.default_rng(12).standard_normal(f.shape))
    fs, es, ehs, ws = _run("fp64", fp, fbg, grids, nsteps, dt, nu, pulses, 1000)
    dev = np.linalg.norm(f64 - fbg[None, :])
    err_f = np.linalg.norm(f32 - f64) / dev
    err_e = _rel(eh32, eh64)
    err_w = _rel(w32, w64)
    print("driven wave 64x1024, 4000 steps, FP32 against FP64: f %.3e (of the deviation), e history %.3e, "
          "field energy %.3e, final e %.3e" % (err_f, err_e, err_w, _rel(e32, e64)))
    print("  FP64 from f perturbed by 1e-7: f %.3e, e history %.3e, field energy %.3e"
          % (np.linalg.norm(fs - f64) / dev, _rel(ehs, eh64), _rel(ws, w64)))
    for a in range(0, nsteps, 1000):
        sl = slice(a, a + 1000)
        print("  steps %4d-%4d: e history FP32 %.3e, perturbed FP64 %.3e; field energy FP32 %.3e"
              % (a, a + 999, _rel(eh32[sl], eh64[sl]), _rel(ehs[sl], eh64[sl]), _rel(w32[sl], w64[sl])))
    assert np.isfinite(f32).all() and np.isfinite(eh32).all()
    assert err_w <= 1e-3
    assert err_e <= 5e-3
    assert err_f <= 1e-2


def test_large_two_stream_fp32_against_fp64():
    """The large run's grid and initial state (4096 x 8192, vmax = 8, two
    streams at +-3: background temperature 10, so the collision weight
    c = nu dt v0t^2 / dv^2 is about 13) over 60 steps."""
    nx, nv, k, vmax, dt, nu, nsteps = 4096, 8192, 0.3, 8.0, 0.05, 1e-4, 60
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    dv, v, kv = vo.velocity_axis(vmax, nv)
    m = np.exp(-((v - 3.0) ** 2) / 2.0) + np.exp(-((v + 3.0) ** 2) / 2.0)
    m = m / np.trapezoid(m, dx=dv)
    phi = np.random.default_rng(4).uniform(0.0, 2 * np.pi, 16)
    pert = 1e-3 * sum(np.cos(mm * k * x + phi[mm - 1]) for mm in range(1, 17))
    f = m[None, :] * (1.0 + pert)[:, None]
    fbg = f.mean(axis=0)
    grids = (x, v, kx, kv, inv, dx, dv)
    f64, e64, eh64, w64 = _run("fp64", f, fbg, grids, nsteps, dt, nu, [], nsteps)
    f32, e32, eh32, w32 = _run("fp32-deltaf", f, fbg, grids, nsteps, dt, nu, [], nsteps)
    err_f = _rel(f32, f64) * np.linalg.norm(f64) / np.linalg.norm(f64 - fbg[None, :])
    err_e = _rel(eh32, eh64)
    err_w = _rel(w32, w64)
    print("two-stream 4096x8192, %d steps: f %.3e (of the deviation), e history %.3e, "
          "field energy %.3e, final e %.3e" % (nsteps, err_f, err_e, err_w, _rel(e32, e64)))
    assert np.isfinite(f32).all()
    assert err_f <= 1e-4
    assert err_e <= 1e-4
    assert err_w <= 1e-4

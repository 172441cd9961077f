"""Failure detection without a GPU fault: the status words that plans,
batches and sweeps raise on the device.

- A field solve that produces NaN or Inf sets VG_FLAG_NONFINITE; the status
  calls report it as VG_ERR_NUMERIC.  The fault is injected on the host: one
  NaN in an otherwise valid state made on the CPU.
- A bounded wait that runs out sets VG_FLAG_TIMEOUT and ends its CTA; the
  sweep's status reports VG_ERR_TIMEOUT.  The test makes the TMA x-drift's
  tile waits wait for tiles nobody requested (a test hook), with a 1 ms
  limit, then checks that the context still works for a new sweep.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import vlapy_oracle as vo  # noqa: E402

pytestmark = pytest.mark.gpu

VG_FLAG_TIMEOUT, VG_FLAG_NONFINITE = 1, 2


@pytest.fixture(scope="module", autouse=True)
def _lib_loaded():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import _lib
    _lib.load()


def _plan(nx, nv, precision="fp64", f_bg=None):
    from vlapy_gb300.plan import Plan
    k = 0.3
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    dv, v, kv = vo.velocity_axis(6.4, nv)
    p = Plan(nx, nv, x, v, kx, kv, inv, dx, dv, dt=0.1, nu=1e-3, collision="dg", precision=precision,
             f_background=f_bg)
    f = vo.maxwellian(nx, nv, 6.4) * (1.0 + 1e-3 * np.cos(k * x))[:, None]
    return p, f


@pytest.mark.parametrize("precision", ["fp64", "fp32-deltaf"])
def test_plan_reports_a_nonfinite_field(precision):
    from vlapy_gb300._lib import VG_ERR_NUMERIC, VlagpuError
    nx, nv = 32, 256
    for poison in (False, True):
        f_bg = vo.maxwellian(1, nv, 6.4)[0] if precision == "fp32-deltaf" else None
        p, f = _plan(nx, nv, precision, f_bg)
        if precision == "fp32-deltaf":
            g = (f - f_bg[None, :]).astype(np.float32)
            if poison:
                g[5, 100] = np.nan
            state = torch.as_tensor(g, device="cuda")
        else:
            if poison:
                f[5, 100] = np.nan
            state = torch.as_tensor(f, device="cuda")
        e = torch.zeros(nx, dtype=torch.float64, device="cuda")
        tb = torch.as_tensor(0.1 * np.arange(3), device="cuda")
        p.run_steps(state, e, None, tb, None, 0, 3, use_graph=False)
        if poison:
            with pytest.raises(VlagpuError) as err:
                p.status()
            assert err.value.status == VG_ERR_NUMERIC
        else:
            assert p.status() == 0
            assert torch.isfinite(e).all()
        p.close()


def test_batch_reports_a_nonfinite_field():
    from vlapy_gb300._lib import VG_ERR_NUMERIC, VlagpuError
    from vlapy_gb300.batch import Batch64
    runs = [dict(nx=32, nv=256, k=0.3, amplitude=1e-3, nu=1e-3), dict(nx=64, nv=512, k=0.35, amplitude=1e-3, nu=0.0)]
    b = Batch64(runs)
    f, e = b.initial_state()
    b.run_steps(f, e, 2)
    assert b.status() == 0
    b.f_of(f, 1)[3, 7] = float("inf")
    b.run_steps(f, e, 2)
    with pytest.raises(VlagpuError) as err:
        b.status()
    assert err.value.status == VG_ERR_NUMERIC
    b.close()


def test_sweep_reports_a_nonfinite_field():
    from vlapy_gb300._lib import VG_ERR_NUMERIC, VlagpuError
    from vlapy_gb300.sweep import Sweep, sweep_config
    sw = Sweep(sweep_config(40, seed=2))
    sw.reset()
    sw.run_steps(2)
    assert sw.status()[0] == 0
    g, e = sw.get_state()
    g[int(sw.g_offsets[17]) + 5] = float("nan")
    sw.set_state(g, e)
    sw.run_steps(2)
    with pytest.raises(VlagpuError) as err:
        sw.status()
    assert err.value.status == VG_ERR_NUMERIC
    sw.close()


def test_sweep_tile_waits_that_run_out_are_reported():
    from vlapy_gb300._lib import VG_ERR_TIMEOUT, VlagpuError
    from vlapy_gb300.sweep import Sweep, sweep_config
    runs = sweep_config(600, seed=4)
    sw = Sweep(runs)
    assert sw.status() == (0, True)  # the x-drift is TMA-fed
    sw.reset()
    sw.set_wait_limit(1_000_000)  # 1 ms
    sw.inject_lost_tiles(True)    # no tile is ever requested: every wait runs out
    sw.run_steps(2)
    with pytest.raises(VlagpuError) as err:
        sw.status()
    assert err.value.status == VG_ERR_TIMEOUT
    sw.close()
    # the context is still usable: a new sweep steps normally
    ok = Sweep(runs)
    ok.reset()
    eh, _ = ok.history(3)
    ok.run_steps(3, eh)
    assert ok.status() == (0, True)
    assert torch.isfinite(eh).all()
    ok.close()

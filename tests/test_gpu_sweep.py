"""Batched sweep (vg_sweep_*) against the FP64 oracle, run by run."""

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


def mixed_runs():
    """All nine shape classes of the sweep workload plus a collisionless run."""
    runs = []
    rng = np.random.default_rng(7)
    for nx in (32, 64, 128):
        for nv in (256, 512, 1024):
            runs.append(dict(nx=nx, nv=nv, k=float(rng.uniform(0.25, 0.45)),
                             amplitude=float(10 ** rng.uniform(-4, -2)),
                             nu=float(10 ** rng.uniform(-5, -2))))
    runs[4]["nu"] = 0.0
    runs.append(dict(nx=32, nv=256, k=0.3, amplitude=1e-6, nu=0.0))
    return runs


def oracle_run(r, nsteps, vmax=6.4, dt=0.1, operator="dg"):
    nx, nv, k = r["nx"], r["nv"], r["k"]
    run = vo.OracleRun(nx, nv, 2 * np.pi / k, vmax, dt, nu=r["nu"], operator=operator)
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    f = vo.maxwellian(nx, nv, vmax) * (1.0 + r["amplitude"] * np.cos(k * x))[:, None]
    f0 = vo.maxwellian(1, nv, vmax)[0]
    e = np.zeros(nx)
    es = []
    for i in range(nsteps):
        e, f = run.step(e, f, dt * i)
        es.append(e)
    return f, np.array(es), f0


def test_sweep_runs_match_oracle():
    from vlapy_gb300.sweep import Sweep
    runs = mixed_runs()
    sw = Sweep(runs)
    sw.reset()
    nsteps = 20
    eh, sh = sw.history(nsteps)
    sw.run_steps(nsteps, eh, sh)
    torch.cuda.synchronize()
    for i, r in enumerate(runs):
        f_ref, e_ref, f0 = oracle_run(r, nsteps)
        f, e = sw.read_run(i)
        f = f.cpu().numpy()
        dev = np.linalg.norm(f - f_ref) / np.linalg.norm(f_ref - f0[None, :])
        assert dev <= 1e-4, (i, r, dev)
        e_hist = sw.e_of(eh, i).cpu().numpy()
        assert np.linalg.norm(e_hist - e_ref) / np.linalg.norm(e_ref) <= 1e-4, (i, r)
        # series: mean density and field energy of the last step
        s_last = sh[-1, i].cpu().numpy()
        np.testing.assert_allclose(s_last[3], np.mean(e_ref[-1] ** 2), rtol=2e-4)
        dv = 2 * 6.4 / r["nv"]
        np.testing.assert_allclose(s_last[0], np.mean(vo.trapz(f_ref, dv, 1)), rtol=1e-9)


def test_sweep_graph_equals_direct():
    from vlapy_gb300.sweep import Sweep
    runs = mixed_runs()
    a, b = Sweep(runs), Sweep(runs)
    a.reset()
    b.reset()
    ea, sa = a.history(8)
    eb, sb = b.history(8)
    a.run_steps(8, ea, sa)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # pool streams do not wait for the default stream
    with torch.cuda.stream(s):
        b.run_steps(8, eb, sb, use_graph=True, stream=s)
    torch.cuda.synchronize()
    # NaN-aware equality: mean f log f is NaN wherever f < 0 in the far tails,
    # as in the reference
    np.testing.assert_array_equal(ea.cpu().numpy(), eb.cpu().numpy())
    np.testing.assert_array_equal(sa.cpu().numpy(), sb.cpu().numpy())
    for i in range(len(runs)):
        np.testing.assert_array_equal(a.read_run(i)[0].cpu().numpy(), b.read_run(i)[0].cpu().numpy())


def test_sweep_tma_x_drift_equals_plain_loads():
    """The x-drift fed by the tensor-memory accelerator (the default for runs
    that start on whole rows) gives the plain-load kernel's result to FP32
    rounding: only the way the tiles reach the transform differs (the two
    kernels may contract their products into FMAs differently).  More runs
    than SMs exercise the persistent CTAs' double-buffered stages."""
    import os
    from vlapy_gb300.sweep import Sweep, sweep_config
    runs = mixed_runs() + sweep_config(600, seed=3)
    a = Sweep(runs)
    os.environ["VG_SWEEP_NO_TMA"] = "1"
    try:
        b = Sweep(runs)
    finally:
        del os.environ["VG_SWEEP_NO_TMA"]
    assert a.status() == (0, True)
    assert b.status() == (0, False)
    for sw in (a, b):
        sw.reset()
    ea, sa = a.history(6)
    eb, sb = b.history(6)
    a.run_steps(6, ea, sa)
    b.run_steps(6, eb, sb)
    torch.cuda.synchronize()
    assert a.status()[0] == 0
    ea, eb = ea.cpu().numpy(), eb.cpu().numpy()
    assert np.isfinite(ea).all()
    assert np.linalg.norm(ea - eb) <= 1e-6 * np.linalg.norm(eb)
    ga, _ = a.get_state()
    gb, _ = b.get_state()
    assert float(torch.linalg.norm((ga - gb).double())) <= 1e-6 * float(torch.linalg.norm(gb.double()))


def test_sweep_classes_side_by_side_equal_serial():
    """The size classes of each phase launched side by side (branches from
    the caller's stream, the default) give bit for bit what one stream gives
    (VG_SWEEP_SERIAL=1), directly and through the captured graph: each class
    works on its own runs."""
    import os
    from vlapy_gb300.sweep import Sweep, sweep_config
    runs = mixed_runs() + sweep_config(300, seed=11)
    a = Sweep(runs)
    os.environ["VG_SWEEP_SERIAL"] = "1"
    try:
        b = Sweep(runs)
    finally:
        del os.environ["VG_SWEEP_SERIAL"]
    for use_graph in (False, True):
        for sw in (a, b):
            sw.reset()
        ea, sa = a.history(5)
        eb, sb = b.history(5)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            a.run_steps(5, ea, sa, use_graph=use_graph, stream=s)
            b.run_steps(5, eb, sb, use_graph=use_graph, stream=s)
        torch.cuda.synchronize()
        assert torch.isfinite(ea).all()
        assert torch.equal(ea, eb)
        torch.testing.assert_close(sa, sb, rtol=0, atol=0, equal_nan=True)
        assert torch.equal(a.get_state()[0], b.get_state()[0])


@pytest.mark.parametrize("use_graph", [False, True])
def test_sweep_step_events_stream_rows_out(use_graph):
    """Step events: one run_steps call records a caller event after each
    step's history row is stored, so a copy stream can take row k to the host
    while the later steps run.  Every row copied that way equals the final
    history, and the events change nothing in the results.  With a graph the
    call is made twice (the capture's launch, then a replay): the events are
    recorded by the graph itself, on every replay."""
    from vlapy_gb300.sweep import Sweep
    runs = mixed_runs()
    a, b = Sweep(runs), Sweep(runs)
    for sw in (a, b):
        sw.reset()
    n = 6
    ea, sa = a.history(n)
    eb, sb = b.history(n)
    events = [torch.cuda.Event() for _ in range(n)]
    a.set_step_events(events)
    stream, copy_stream = torch.cuda.Stream(), torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    host_e = torch.zeros((n, a.x_points), dtype=torch.float64).pin_memory()
    host_s = torch.zeros((n, a.n_runs, 7), dtype=torch.float64).pin_memory()
    for _ in range(2 if use_graph else 1):
        with torch.cuda.stream(stream):
            a.run_steps(n, ea, sa, use_graph=use_graph, stream=stream)
        for k in range(n):
            copy_stream.wait_event(events[k])
            with torch.cuda.stream(copy_stream):
                host_e[k].copy_(ea[k], non_blocking=True)
                host_s[k].copy_(sa[k], non_blocking=True)
        b.run_steps(n, eb, sb)
        torch.cuda.synchronize()
        assert torch.equal(host_e, ea.cpu()) and torch.equal(ea, eb)
        torch.testing.assert_close(host_s, sa.cpu(), rtol=0, atol=0, equal_nan=True)
        torch.testing.assert_close(sa, sb, rtol=0, atol=0, equal_nan=True)
    a.set_step_events([])
    assert torch.equal(a.get_state()[0], b.get_state()[0])


def test_sweep_config_distribution():
    from vlapy_gb300.sweep import sweep_config
    runs = sweep_config(4096)
    nx = np.array([r["nx"] for r in runs])
    nu = np.array([r["nu"] for r in runs])
    assert set(nx) == {32, 64, 128}
    assert 0.2 < np.mean(nu == 0.0) < 0.3
    assert all(0.25 <= r["k"] <= 0.45 for r in runs)
    assert all(1e-6 <= r["amplitude"] <= 1e-2 for r in runs)


def test_sweep_landau_rates():
    """Collisionless runs of the sweep damp at the oracle's rate (within 1%)."""
    from vlapy_gb300.sweep import Sweep
    ks = (0.3, 0.35, 0.4)
    runs = [dict(nx=32, nv=512, k=k, amplitude=1e-4, nu=0.0) for k in ks]
    sw = Sweep(runs)
    sw.reset()
    nsteps = 600
    eh, sh = sw.history(nsteps)
    sw.run_steps(nsteps, eh, sh)
    torch.cuda.synchronize()
    t = 0.1 * np.arange(1, nsteps + 1)
    for i, r in enumerate(runs):
        _, e_ref, _ = oracle_run(r, nsteps)
        a_gpu = vo.mode_amplitude(sw.e_of(eh, i).cpu().numpy())
        a_ref = vo.mode_amplitude(e_ref)
        rg, wg = vo.envelope_fit(t, a_gpu, t_min=5.0)
        rr, wr = vo.envelope_fit(t, a_ref, t_min=5.0)
        assert abs(rg - rr) <= 0.01 * abs(rr), (r, rg, rr)
        assert abs(wg - wr) <= 0.01 * abs(wr), (r, wg, wr)


def test_sweep_rejects_unsupported_shapes():
    from vlapy_gb300.sweep import Sweep
    with pytest.raises(NotImplementedError):
        Sweep([dict(nx=48, nv=256, k=0.3, amplitude=1e-3, nu=0.0)])
    with pytest.raises(NotImplementedError):
        Sweep([dict(nx=8, nv=64, k=0.3, amplitude=1e-3, nu=0.0)])


def test_sweep_reset_after_steps_equals_fresh():
    """reset() clears the field and its FP32 copy: a reused sweep repeats a fresh one bit for bit."""
    from vlapy_gb300.sweep import Sweep
    runs = mixed_runs()
    a, b = Sweep(runs), Sweep(runs)
    a.reset()
    a.run_steps(7)
    a.reset()
    b.reset()
    ea, sa = a.history(5)
    eb, sb = b.history(5)
    a.run_steps(5, ea, sa)
    b.run_steps(5, eb, sb)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ea.cpu().numpy(), eb.cpu().numpy())
    ga, gb = a.get_state()[0], b.get_state()[0]
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ga.cpu().numpy(), gb.cpu().numpy())


def test_sweep_state_moves_between_sweeps():
    """get_state / set_state: 6 + 6 steps through a second sweep equal 12 steps of one."""
    from vlapy_gb300.sweep import Sweep
    runs = mixed_runs()
    a, b, c = Sweep(runs), Sweep(runs), Sweep(runs)
    for s in (a, b, c):
        s.reset()
    a.run_steps(12)
    b.run_steps(6)
    g, e = b.get_state()
    c.set_state(g, e)
    c.run_steps(6)
    torch.cuda.synchronize()
    ga, ea = a.get_state()
    gc, ec = c.get_state()
    torch.cuda.synchronize()
    assert g.shape == (a.cells,) and e.shape == (a.x_points,)
    # the split run applies the two half-kicks at step 6 as separate passes
    assert torch.linalg.norm(gc - ga) <= 1e-5 * torch.linalg.norm(ga)
    assert torch.linalg.norm(ec - ea) <= 1e-5 * torch.linalg.norm(ea)


def test_sweep_damping_on_device_matches_host_fit():
    """vg_sweep_damping equals the host diagnostic on the same histories."""
    from vlapy_gb300.diagnostics import damping_fit, mode_amplitude
    from vlapy_gb300.sweep import Sweep
    runs = mixed_runs()
    sw = Sweep(runs)
    sw.reset()
    nsteps = 400
    eh, sh = sw.history(nsteps)
    sw.run_steps(nsteps, eh, sh)
    t = 0.1 * np.arange(1, nsteps + 1)
    for t_min, t_max in ((5.0, 40.0), (5.0, None), (30.0, 30.4)):
        rate, freq = sw.damping(eh, t_min=t_min, t_max=t_max)
        rate, freq = rate.cpu().numpy(), freq.cpu().numpy()
        for i in range(len(runs)):
            rh, fh = damping_fit(t, mode_amplitude(sw.e_of(eh, i).cpu().numpy()), t_min=t_min, t_max=t_max)
            if np.isnan(rh):
                assert np.isnan(rate[i]) and np.isnan(freq[i]), (i, t_min, t_max)
            else:
                np.testing.assert_allclose(rate[i], rh, rtol=1e-7, atol=1e-12)
                np.testing.assert_allclose(freq[i], fh, rtol=1e-9)
    with pytest.raises(ValueError):
        sw.damping(eh[:, :5].contiguous())


@pytest.mark.parametrize("nx,nv", [(8, 512), (256, 64), (16, 2048), (256, 256), (128, 2048)])
def test_sweep_extreme_shapes_match_oracle(nx, nv):
    """The smallest and largest supported nx and nv of a sweep class (nx in
    [8, 256], nv in [64, 2048], nv >= 4096 / nx), alone and beside another class."""
    from vlapy_gb300.sweep import Sweep
    runs = [dict(nx=nx, nv=nv, k=0.35, amplitude=1e-3, nu=1e-3), dict(nx=32, nv=256, k=0.3, amplitude=1e-2, nu=0.0)]
    sw = Sweep(runs)
    sw.reset()
    sw.run_steps(5)
    torch.cuda.synchronize()
    for i, r in enumerate(runs):
        f_ref, _, f0 = oracle_run(r, 5)
        f = sw.read_run(i)[0].cpu().numpy()
        assert np.linalg.norm(f - f_ref) / np.linalg.norm(f_ref - f0[None, :]) <= 1e-4, (nx, nv, i)


def test_sweep_lenard_bernstein_matches_oracle():
    """The sweep with the Lenard-Bernstein operator (vlapy/core/collisions.py:26-83)."""
    from vlapy_gb300.sweep import Sweep
    runs = [dict(nx=32, nv=512, k=0.3, amplitude=1e-3, nu=5e-3), dict(nx=64, nv=256, k=0.4, amplitude=1e-2, nu=1e-2)]
    sw = Sweep(runs, collision="lb")
    sw.reset()
    sw.run_steps(10)
    torch.cuda.synchronize()
    for i, r in enumerate(runs):
        f_ref, _, f0 = oracle_run(r, 10, operator="lb")
        f = sw.read_run(i)[0].cpu().numpy()
        assert np.linalg.norm(f - f_ref) / np.linalg.norm(f_ref - f0[None, :]) <= 1e-4, (i, r)


def test_sweep_full_size_properties():
    """The default workload at its full size (4096 runs, 1.8e8 cells), through
    properties that do not depend on the size: everything finite, each run's
    density conserved, each run's result independent of the batch it ran in
    (bit for bit), and one run of each shape class against the oracle."""
    from vlapy_gb300.sweep import Sweep, sweep_config
    runs = sweep_config(4096, 20261203)
    nsteps = 20
    sw = Sweep(runs)
    sw.reset()
    eh, sh = sw.history(nsteps)
    sw.run_steps(nsteps, eh, sh)
    torch.cuda.synchronize()
    assert torch.isfinite(eh).all() and torch.isfinite(sh[:, :, :4]).all()
    # density (n ~ 1): kicks and drifts keep it exactly, the collision keeps it
    # discretely; FP32 delta-f rounding (~1e-7 of |g| <= 1e-2 a step) moves it
    # by ~1e-9 over these steps
    n = sh[:, :, 0].cpu().numpy()
    assert np.abs(n - n[:1]).max() <= 1e-8
    # batching independence: every 7th run in a sweep of its own
    idx = list(range(0, len(runs), 7))
    sub = Sweep([runs[i] for i in idx])
    sub.reset()
    eb, sb = sub.history(nsteps)
    sub.run_steps(nsteps, eb, sb)
    torch.cuda.synchronize()
    # (mean f log f is NaN where f < 0 in the far tails, as in the reference)
    torch.testing.assert_close(sh[:, idx, :], sb, rtol=0, atol=0, equal_nan=True)
    for j, i in enumerate(idx[::37]):
        assert torch.equal(sw.e_of(eh, i), sub.e_of(eb, j * 37))
        assert torch.equal(sw.read_run(i)[0], sub.read_run(j * 37)[0])
    # one run of each (nx, nv) class against the FP64 oracle
    seen = set()
    for i, r in enumerate(runs):
        key = (r["nx"], r["nv"])
        if key in seen:
            continue
        seen.add(key)
        f_ref, e_ref, f0 = oracle_run(r, nsteps)
        f = sw.read_run(i)[0].cpu().numpy()
        assert np.linalg.norm(f - f_ref) / np.linalg.norm(f_ref - f0[None, :]) <= 1e-4, (i, r)
        e_hist = sw.e_of(eh, i).cpu().numpy()
        assert np.linalg.norm(e_hist - e_ref) / np.linalg.norm(e_ref) <= 1e-4, (i, r)
    assert len(seen) == 9


def test_sweep_full_horizon_against_fp64():
    """The benchmarked horizon (2000 steps) of the sweep workload, 16 runs of
    each of the nine shape classes drawn from the workload's own run list
    (collisional and collisionless), against the batched FP64 step (the
    reference's arithmetic, held to the oracle at 1e-12 in test_gpu_batch):
    each run's Landau damping rate (peak-envelope fit of |E_1| on t in [5, 60])
    within 1 %, its field-energy history within 1 %, and its final f within
    a stated bound of the perturbation."""
    from vlapy_gb300.batch import Batch64
    from vlapy_gb300.diagnostics import damping_fit, mode_amplitude
    from vlapy_gb300.sweep import Sweep, sweep_config
    pool = sweep_config(4096, 20261203)
    runs, count = [], {}
    for r in pool:
        key = (r["nx"], r["nv"])
        if count.get(key, 0) < 16:
            count[key] = count.get(key, 0) + 1
            runs.append(r)
    assert len(runs) == 144 and any(r["nu"] == 0.0 for r in runs) and any(r["nu"] > 0.0 for r in runs)
    nsteps = 2000
    sw = Sweep(runs)
    sw.reset()
    eh, sh = sw.history(nsteps)
    sw.run_steps(nsteps, eh, sh)
    ref64 = Batch64(runs)
    f64, e64 = ref64.initial_state()
    eh64, sh64 = ref64.history(nsteps)
    for c0 in range(0, nsteps, 250):
        ref64.run_steps(f64, e64, 250, eh64, sh64, row0=c0)
    torch.cuda.synchronize()
    t = 0.1 * np.arange(1, nsteps + 1)
    rate_err, e2_err, f_err = [], [], []
    for i, r in enumerate(runs):
        rf, _ = damping_fit(t, mode_amplitude(ref64.e_of(eh64, i).cpu().numpy()), t_min=5.0, t_max=60.0)
        rg, _ = damping_fit(t, mode_amplitude(sw.e_of(eh, i).cpu().numpy()), t_min=5.0, t_max=60.0)
        assert np.isfinite(rf) and rf < 0.0, (i, r, rf)
        rate_err.append(abs(rg - rf) / abs(rf))
        e2_ref = ref64.series_of(sh64, i)[:, 3].cpu().numpy()
        e2 = sh[:, i, 3].cpu().numpy()
        e2_err.append(np.linalg.norm(e2 - e2_ref) / np.linalg.norm(e2_ref))
        f_ref = ref64.f_of(f64, i).cpu().numpy()
        f0 = vo.maxwellian(1, r["nv"], 6.4)[0]
        f_err.append(np.linalg.norm(sw.read_run(i)[0].cpu().numpy() - f_ref) / np.linalg.norm(f_ref - f0[None, :]))
    rate_err, e2_err, f_err = map(np.asarray, (rate_err, e2_err, f_err))
    print("horizon 2000 steps, 144 runs: damping rate rel err median %.2e max %.2e; field energy median %.2e "
          "max %.2e; final f (of |f - f0|) median %.2e max %.2e"
          % (np.median(rate_err), rate_err.max(), np.median(e2_err), e2_err.max(), np.median(f_err), f_err.max()))
    assert rate_err.max() <= 0.01, (int(rate_err.argmax()), runs[int(rate_err.argmax())])
    assert e2_err.max() <= 0.01, (int(e2_err.argmax()), runs[int(e2_err.argmax())])
    assert f_err.max() <= 0.02, (int(f_err.argmax()), runs[int(f_err.argmax())])
    ref64.close()


def test_sweep_full_workload_full_horizon():
    """The benchmarked workload itself, all 4096 runs over their 2000 steps
    (one graph replay): no bounded wait ran out and no field went non-finite,
    every stored field is finite, every run's density is conserved, and one
    run of each (nx, nv) class (collisional and collisionless where the class
    has both) damps at the batched FP64 step's rate within 1 %."""
    from vlapy_gb300.batch import Batch64
    from vlapy_gb300.diagnostics import damping_fit, mode_amplitude
    from vlapy_gb300.sweep import Sweep, sweep_config
    runs = sweep_config(4096, 20261203)
    nsteps = 2000
    sw = Sweep(runs)
    sw.reset()
    eh, sh = sw.history(nsteps)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        sw.run_steps(nsteps, eh, sh, use_graph=True, stream=s)
    torch.cuda.synchronize()
    assert sw.status() == (0, True)
    assert torch.isfinite(eh).all() and torch.isfinite(sh[:, :, :4]).all()
    n = sh[:, :, 0]
    drift = float(((n - n[:1]).abs() / n[:1].abs()).max())
    assert drift <= 1e-6, drift
    # one collisional and one collisionless run of each shape class
    picked, seen = [], set()
    for i, r in enumerate(runs):
        key = (r["nx"], r["nv"], r["nu"] == 0.0)
        if key not in seen:
            seen.add(key)
            picked.append(i)
    assert len(picked) >= 18
    ref64 = Batch64([runs[i] for i in picked])
    f64, e64 = ref64.initial_state()
    eh64, _ = ref64.history(nsteps)
    for c0 in range(0, nsteps, 500):
        ref64.run_steps(f64, e64, 500, eh64, None, row0=c0)
    torch.cuda.synchronize()
    t = 0.1 * np.arange(1, nsteps + 1)
    for j, i in enumerate(picked):
        rf, _ = damping_fit(t, mode_amplitude(ref64.e_of(eh64, j).cpu().numpy()), t_min=5.0, t_max=60.0)
        rg, _ = damping_fit(t, mode_amplitude(sw.e_of(eh, i).cpu().numpy()), t_min=5.0, t_max=60.0)
        assert np.isfinite(rf) and abs(rg - rf) <= 0.01 * abs(rf), (i, runs[i], rg, rf)
    ref64.close()
    sw.close()


def test_profile_records_the_last_row_pass_apart():
    """The per-kernel record of a 3-step call: one leading half kick, three
    x-drifts, field solves and stores, two row passes that end with the next
    step's leading half kick, and the last step's row pass (without it) under
    its own name."""
    from vlapy_gb300.sweep import Sweep
    sw = Sweep(mixed_runs())
    sw.reset()
    eh, sh = sw.history(3)
    sw.profile(True)
    sw.run_steps(3, eh, sh)
    prof = sw.profile_read()
    sw.profile(False)
    assert {k: v["launches"] for k, v in prof.items()} == {
        "sweep_kick": 1, "sweep_x_drift": 3, "sweep_field": 3, "sweep_row_pass": 2, "sweep_store": 3,
        "sweep_row_pass_last": 1}
    assert all(v["total_ms"] > 0 for v in prof.values())
    sw.close()

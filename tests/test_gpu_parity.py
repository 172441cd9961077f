"""FP64 GPU path against the CPU oracle and the reference's golden vectors.

Bar: relative L2 <= 1e-12 for f and e per step; the trapz densities and the
Fokker-Planck solve reproduce NumPy's rounding and are checked bit for bit.
All calls go through libvlagpu.so (the C ABI) via the vlapy_gb300 host layer.
"""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import vlapy_oracle as vo  # noqa: E402

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-12


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module", autouse=True)
def _lib_loaded():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import _lib
    _lib.load()


def make_plan(nx, nv, k=0.3, vmax=6.4, dt=0.1, nu=0.0, collision="none", integrator="leapfrog",
              pulses=None):
    from vlapy_gb300.plan import Plan
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    dv, v, kv = vo.velocity_axis(vmax, nv)
    p = Plan(nx, nv, x, v, kx, kv, inv, dx, dv, dt=dt, nu=nu, collision=collision,
             integrator=integrator, pulses=pulses)
    return p, (x, v, kx, kv, inv, dx, dv)


def perturbed(nx, nv, k=0.3, vmax=6.4, amp=1e-2, seed=0):
    rng = np.random.default_rng(seed)
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    f = vo.maxwellian(nx, nv, vmax)
    pert = np.zeros(nx)
    for m in range(1, min(4, nx // 2 + 1)):
        pert += amp * rng.uniform(0.2, 1.0) * np.cos(m * k * x + rng.uniform(0, 2 * np.pi))
    return f * (1.0 + pert)[:, None]


def cuda(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


SHAPES = [(32, 512), (16, 128), (7, 64), (64, 1024), (2, 8192), (4, 2), (256, 32), (8192, 4),
          (4096, 8), (12, 96), (5, 1000), (96, 30), (3, 4095)]


@pytest.mark.parametrize("nx,nv", SHAPES)
def test_edfdv_matches_oracle(nx, nv):
    p, (x, v, kx, kv, inv, dx, dv) = make_plan(nx, nv)
    f = perturbed(nx, nv)
    e = 0.05 * np.sin(0.3 * x) + 0.01
    for dt in (0.05, 0.1, -0.37):
        ref = vo.edfdv_exponential(f, e, kv, dt)
        g = cuda(f)
        p.edfdv(g, cuda(e), dt)
        assert rel(g.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("nx,nv", SHAPES)
def test_vdfdx_matches_oracle(nx, nv):
    p, (x, v, kx, kv, inv, dx, dv) = make_plan(nx, nv)
    f = perturbed(nx, nv)
    for dt in (0.1, 0.05, 1.3):
        ref = vo.vdfdx_exponential(f, kx, v, dt)
        g = cuda(f)
        p.vdfdx(g, dt)
        assert rel(g.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("nx,nv", [(32, 512), (7, 64), (3, 1000), (64, 1024), (2, 8192), (5, 9)])
def test_charge_density_bit_exact(nx, nv):
    p, (x, v, kx, kv, inv, dx, dv) = make_plan(nx, 2 if nv < 2 else nv)
    f = perturbed(nx, nv) if nv >= 2 else None
    out = torch.empty(nx, dtype=torch.float64, device="cuda")
    p.charge_density(cuda(f), out)
    np.testing.assert_array_equal(out.cpu().numpy(), vo.charge_density(f, dv))


def test_poisson_golden_any_nx():
    """nx = 96 (not a power of two): the reference's analytic field test."""
    d = np.load(os.path.join(G, "poisson_96.npz"))
    from vlapy_gb300.core import field
    for i in range(3):
        # e = solve_for_field(charge) = __fft_solve__(1 - charge)
        got = field.__fft_solve__(cuda(1.0 - d["charge"][i]), d["one_over_kx"]).cpu().numpy()
        assert rel(got, d["e"][i]) <= TOL
        got2 = field.solve_for_field(cuda(d["charge"][i]), d["one_over_kx"]).cpu().numpy()
        assert rel(got2, d["e"][i]) <= TOL


@pytest.mark.parametrize("nx", [2, 8, 32, 64, 1024, 8192])
def test_field_solve_matches_oracle(nx):
    p, (x, v, kx, kv, inv, dx, dv) = make_plan(nx, 256)
    f = perturbed(nx, 256, amp=1e-4)
    drv = 1e-3 * np.cos(0.3 * x)
    ref = vo.total_field(drv, f, dv, inv)
    out = torch.empty(nx, dtype=torch.float64, device="cuda")
    p.field_solve(cuda(f), cuda(drv), out)
    assert rel(out.cpu().numpy(), ref) <= TOL
    p.field_solve(cuda(f), None, out)
    assert rel(out.cpu().numpy(), vo.total_field(np.zeros(nx), f, dv, inv)) <= TOL


@pytest.mark.parametrize("op", ["lb", "dg"])
@pytest.mark.parametrize("vs", [0.0, 0.5, 1.5])
def test_collisions_golden_bit_exact(op, vs):
    """tests/test_collisions.py parameters: nx=2, nv=1024, nu=1e-2, dt=0.1;
    the GPU diagonals and Thomas recurrence follow the reference operation
    for operation, so the result is bit-identical."""
    d = np.load(os.path.join(G, "collisions_2x1024.npz"))
    tag = "%s_vs%g" % (op, vs)
    from vlapy_gb300.core import step
    nv, vmax = 1024, 6.0
    dv = 2 * vmax / nv
    v = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    stuff = {"f": d["fin_" + tag], "v": v, "nv": nv, "nx": 2, "nu": 1e-2, "dt": 0.1, "dv": dv}
    params = {"fokker-planck": {"type": op, "solver": "batched_tridiagonal"}, "nu": 1e-2}
    fp = step.get_collision_step(stuff, params)
    g = cuda(d["fin_" + tag])
    for it in range(16):
        g = fp(g)
        if it == 0:
            np.testing.assert_array_equal(g.cpu().numpy(), d["f1_" + tag])
    np.testing.assert_array_equal(g.cpu().numpy(), d["f16_" + tag])


@pytest.mark.parametrize("op", ["lb", "dg"])
def test_collision_physics(op):
    """The reference's own conservation checks (tests/test_collisions.py:39-165)."""
    from vlapy_gb300.core import step
    nv, vmax = 1024, 6.0
    dv = 2 * vmax / nv
    v = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    for vs in (0.0, 0.5, 1.5):
        f = vo.shifted_maxwellian(2, v, 1.0, vs)
        stuff = {"f": f, "v": v, "nv": nv, "nx": 2, "nu": 1e-2, "dt": 0.1, "dv": dv}
        fp = step.get_collision_step(stuff, {"fokker-planck": {"type": op, "solver": "batched_tridiagonal"},
                                             "nu": 1e-2})
        g = cuda(f)
        for _ in range(16):
            g = fp(g)
        out = g.cpu().numpy()
        if vs == 0.0:
            np.testing.assert_almost_equal(f, out, decimal=4)
            np.testing.assert_almost_equal(vo.trapz(f * v, dv, 1), vo.trapz(out * v, dv, 1), decimal=4)
        if vs == 0.5:
            np.testing.assert_almost_equal(vo.trapz(out, dv, 1), vo.trapz(f, dv, 1), decimal=4)
            np.testing.assert_almost_equal(vo.trapz(out * v ** 2, dv, 1), vo.trapz(f * v ** 2, dv, 1), decimal=4)
        if vs == 1.5:
            jin, jout = vo.trapz(f * v, dv, 1), vo.trapz(out * v, dv, 1)
            if op == "lb":
                assert np.all(jout < jin)
            else:
                np.testing.assert_almost_equal(jin, jout, decimal=4)


def _golden_run(name):
    from vlapy_gb300 import field_driver
    from vlapy_gb300.core import step
    from vlapy_gb300.outer_loop import get_arrays_for_inner_loop
    d = np.load(os.path.join(G, name + ".npz"))
    m = {k[5:]: d[k][()] for k in d.files if k.startswith("meta_")}
    nx, nv = int(m["nx"]), int(m["nv"])
    xmax, vmax, dt, nu = float(m["xmax"]), float(m["vmax"]), float(m["dt"]), float(m["nu"])
    n_modes = int(m["n_modes"])
    dx, x, kx, inv = vo.spatial_axis(0.0, xmax, nx)
    dv, v, kv = vo.velocity_axis(vmax, nv)
    drv = None
    if "pulse_k0" in d.files:
        pulses = {"p": {k: float(d["pulse_" + k]) for k in ("k0", "w0", "a0", "t_L", "t_R", "t_wL", "t_wR")}}
        if "pulse_envelope" in d.files:
            pulses["p"]["envelope"] = str(d["pulse_envelope"])
        drv = field_driver.get_driver_function(x, pulses)
    rules = ({"time": "first-last", "space": "all"} if n_modes < 0
             else {"time": "first-last", "space": ["k%d" % i for i in range(n_modes)]})
    stuff = {"nx": nx, "nv": nv, "x": x, "v": v, "kx": kx, "kv": kv, "one_over_kx": inv, "dv": dv,
             "dt": dt, "nu": nu, "driver_function": drv, "rules_to_store_f": rules,
             "f": d["f0"], "e": np.zeros(nx)}
    params = {"nu": nu, "fokker-planck": {"type": str(m["fp_type"]), "solver": "batched_tridiagonal"},
              "vlasov-poisson": {"time": str(m["time"]), "vdfdx": str(m.get("vdfdx", "exponential")),
                                 "edfdv": str(m.get("edfdv", "exponential")), "poisson": "spectral"},
              "backend": {"core": "gb300", "precision": "fp64"}}
    return d, m, stuff, params, rules, step, get_arrays_for_inner_loop


@pytest.mark.parametrize("name", ["landau_32x512", "driven_dg_16x256", "driven_lb_16x256",
                                  "integrator_pefrl_16x128", "integrator_h-sixth_16x128",
                                  "step_sl_dg_16x64", "step_cd2_16x64", "driven_sin2_dg_64x1024"])
def test_timestep_matches_golden(name):
    """The reference's own time steps, including the driven-wave workload's
    grid (64 x 1024, Dougherty nu = 1e-3) under the sin^2-envelope driver,
    whose pulses the device evaluates at every sub-step time."""
    d, m, stuff, params, rules, step, arrays = _golden_run(name)
    nsteps = int(m["nsteps"])
    ts = step.get_timestep(params, stuff)
    sc = arrays(stuff, nsteps, rules)
    sc["time_batch"] = cuda(d["time"])
    sc["driver_array_batch"] = cuda(d["driver_array"])
    for i in range(nsteps):
        sc, _ = ts(sc, i)
        if "f_%d" % (i + 1) in d.files:
            assert rel(sc["f"].cpu().numpy(), d["f_%d" % (i + 1)]) <= TOL * (i + 1)
            assert rel(sc["e"].cpu().numpy(), d["e_%d" % (i + 1)]) <= TOL * (i + 1)
    _check_storage(sc, d, nsteps)


# velocity power of each stored moment (vlapy/core/step.py:164-171)
FIELD_POW = {"n": 0, "j": 1, "T": 2, "q": 3, "fv4": 4, "vN": 5}


def _check_storage(sc, d, nsteps):
    f0 = d["f0"]
    nx, nv = f0.shape
    vmax = float(d["meta_vmax"])
    dv, v, kv = vo.velocity_axis(vmax, nv)
    # long fixtures keep every ke-th row of the fields other than e, and of stored_f
    ke = int(d["meta_keep_every"]) if "meta_keep_every" in d.files else 1
    # f carries up to TOL relative error per step (the FFT rounding differs from
    # pocketfft's): the bounds on its moments grow with the steps like f's own
    grow = max(1.0, nsteps / 10.0)
    for k in vo.FIELD_KEYS:
        got = sc["fields"][k].cpu().numpy()[::1 if k == "e" else ke]
        ref = d["fields_" + k]
        if k == "driver":
            np.testing.assert_array_equal(got, ref)
        elif k == "e":
            assert rel(got, ref) <= 1e-11 * grow, k
        else:
            # odd moments of a near-symmetric f are ~0: bound the error by the
            # scale of the integrand, trapz(|f| |v|^p)
            scale = vo.trapz(np.abs(f0) * np.abs(v) ** FIELD_POW[k], dv, 1).max()
            np.testing.assert_allclose(got, ref, rtol=1e-11 * grow, atol=1e-12 * scale * grow, err_msg=k)
    for k in vo.SERIES_KEYS:
        got = sc["series"][k].cpu().numpy()
        atol = 1e-14
        if k == "mean_j":
            # the mean current of a near-symmetric f is ~0: bound its error by the
            # scale of the integrand, as for the odd moments above
            atol = max(atol, 1e-12 * vo.trapz(np.abs(f0) * np.abs(v), dv, 1).mean())
        np.testing.assert_allclose(got, d["series_" + k], rtol=1e-11 * grow, atol=atol * grow, err_msg=k)
    sf = sc["stored_f"].cpu().numpy()[::ke]
    ref = d["stored_f"]
    if sf.dtype == np.complex64:
        np.testing.assert_allclose(sf, ref, rtol=2e-6, atol=1e-6 * np.abs(ref).max())
    else:
        assert rel(sf, ref) <= 1e-11


@pytest.mark.parametrize("name", ["landau_32x512", "driven_dg_16x256", "driven_sin2_dg_64x1024"])
def test_inner_loop_graph_matches_golden(name):
    """The graph-captured inner loop over the whole batch."""
    from vlapy_gb300 import outer_loop
    d, m, stuff, params, rules, step, arrays = _golden_run(name)
    nsteps = int(m["nsteps"])
    sc, inner = outer_loop.get_sim_config_and_inner_loop_step(params, stuff, nsteps, rules)
    for rep in range(2):
        if rep == 1:  # replay from the start: same graph, refreshed state
            sc["f"].copy_(cuda(d["f0"]))
            sc["e"].zero_()
            sc["mean_cum_de2_previous"] = 0.0
        sc = inner(d["time"], d["driver_array"], sc)
        torch.cuda.synchronize()
        assert rel(sc["f"].cpu().numpy(), d["f_%d" % nsteps]) <= TOL * nsteps
        assert rel(sc["e"].cpu().numpy(), d["e_%d" % nsteps]) <= TOL * nsteps
        _check_storage(sc, d, nsteps)
        # what StorageManager.batch_update (vlapy/storage.py:177-315) receives
        from vlapy_gb300 import storage
        fields, stored_f, t, series, cur = storage.check_batch(sc, stuff["x"], stuff["v"], rules)
        np.testing.assert_array_equal(t, d["time"])
        assert "mean_cum_de2" in series and stored_f.shape[0] == nsteps


def test_leapfrog_parity_many_steps():
    """100 FP64 steps at the Landau workload's grid against the oracle."""
    nx, nv, k = 32, 512, 0.3
    p, (x, v, kx, kv, inv, dx, dv) = make_plan(nx, nv)
    f0 = vo.maxwellian(nx, nv, 6.4) * (1.0 + 1e-4 * np.cos(k * x))[:, None]
    run = vo.OracleRun(nx, nv, 2 * np.pi / k, 6.4, 0.1)
    e, f = np.zeros(nx), f0
    g, eg = cuda(f0), torch.zeros(nx, dtype=torch.float64, device="cuda")
    tb = cuda(0.1 * np.arange(100))
    p.run_steps(g, eg, None, tb, None, 0, 100, use_graph=False)
    for i in range(100):
        e, f = run.step(e, f, 0.1 * i)
    assert rel(g.cpu().numpy(), f) <= 1e-11
    assert rel(eg.cpu().numpy(), e) <= 1e-10


def test_non_power_of_two_steps_match_oracle():
    """Full steps (leapfrog, Dougherty collisions, storage) on grids that are
    not powers of two, where both advections take the direct-DFT path, against
    the oracle (the reference transforms any length)."""
    nx, nv, k, nu, nsteps = 12, 96, 0.3, 1e-3, 5
    p, (x, v, kx, kv, inv, dx, dv) = make_plan(nx, nv, nu=nu, collision="dg")
    f0 = perturbed(nx, nv, amp=1e-2)
    run = vo.OracleRun(nx, nv, 2 * np.pi / k, 6.4, 0.1, nu=nu, operator="dg")
    e, f = np.zeros(nx), f0
    g, eg = cuda(f0), torch.zeros(nx, dtype=torch.float64, device="cuda")
    tb = cuda(0.1 * np.arange(nsteps))
    p.run_steps(g, eg, None, tb, None, 0, nsteps, use_graph=False)
    for i in range(nsteps):
        e, f = run.step(e, f, 0.1 * i)  # VP step, then the collision step
    assert rel(g.cpu().numpy(), f) <= TOL * nsteps
    assert rel(eg.cpu().numpy(), e) <= TOL * nsteps


def test_unsupported_sizes_raise():
    """Lengths that are not powers of two go through direct DFTs up to 4096;
    longer ones are refused."""
    p, _ = make_plan(4100, 4)
    g = cuda(np.ones((4100, 4)))
    with pytest.raises(NotImplementedError):
        p.vdfdx(g, 0.1)
    p2, _ = make_plan(2, 4100)
    with pytest.raises(NotImplementedError):
        p2.edfdv(cuda(np.ones((2, 4100))), cuda(np.zeros(2)), 0.1)


def test_dropin_fp32_resident_deviation():
    """The reference-facing per-step closure and inner loop in the FP32
    delta-f mode, on the driven-wave fixture: the FP32 deviation g = f - f0
    stays resident between calls (f is written from it once a step and never
    read back), the per-step closure and the graph-captured inner loop agree,
    both follow the reference's FP64 steps to the FP32 mode's error, and a
    caller that writes f restarts from the f it wrote."""
    from vlapy_gb300 import outer_loop
    d, m, stuff, params, rules, step, arrays = _golden_run("driven_sin2_dg_64x1024")
    params = dict(params, backend={"core": "gb300", "precision": "fp32-deltaf"})
    nsteps = int(m["nsteps"])
    ts = step.get_timestep(params, stuff)
    sc = arrays(stuff, nsteps, rules)
    sc["time_batch"] = cuda(d["time"])
    sc["driver_array_batch"] = cuda(d["driver_array"])
    resident, f_after_1 = None, None
    for i in range(nsteps):
        sc, _ = ts(sc, i)
        if i == 0:
            resident = sc["_g"][0]
            f_after_1 = sc["f"].clone()
        assert sc["_g"][0] is resident
    f_step = sc["f"].cpu().numpy()
    sc2, inner = outer_loop.get_sim_config_and_inner_loop_step(params, stuff, nsteps, rules)
    sc2 = inner(d["time"], d["driver_array"], sc2)
    torch.cuda.synchronize()
    f_loop = sc2["f"].cpu().numpy()
    f_ref = d["f_%d" % nsteps]
    pert = np.linalg.norm(f_ref - d["f0"].mean(axis=0)[None, :])
    assert np.linalg.norm(f_step - f_loop) <= 1e-5 * pert
    assert np.linalg.norm(f_step - f_ref) <= 1e-4 * pert
    np.testing.assert_allclose(sc["e"].cpu().numpy(), sc2["e"].cpu().numpy(), rtol=0,
                               atol=1e-5 * np.abs(d["e_%d" % nsteps]).max())
    # the caller writes f (and e): the next step starts from them
    sc["f"].copy_(cuda(d["f0"]))
    sc["e"].zero_()
    sc, _ = ts(sc, 0)
    assert sc["_g"][0] is not resident
    torch.testing.assert_close(sc["f"], f_after_1, rtol=0, atol=0)

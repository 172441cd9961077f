"""Batched FP64 step (vg_batch_*): against single plans bit for bit, against
the oracle, and against the reference's own Landau steps (golden fixture)."""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import vlapy_oracle as vo  # noqa: E402

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _lib_loaded():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import _lib
    _lib.load()


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def mixed_runs():
    """All nine shape classes of the sweep workload, in an order that is not
    grouped by nv, with two collisionless runs."""
    runs = []
    rng = np.random.default_rng(17)
    for nv in (512, 256, 1024):
        for nx in (64, 32, 128):
            runs.append(dict(nx=nx, nv=nv, k=float(rng.uniform(0.25, 0.45)),
                             amplitude=float(10 ** rng.uniform(-4, -2)), nu=float(10 ** rng.uniform(-5, -2))))
    runs[2]["nu"] = 0.0
    runs.append(dict(nx=32, nv=512, k=0.3, amplitude=1e-3, nu=0.0))
    return runs


def _plan_steps(r, nsteps, vmax=6.4, dt=0.1):
    """The same run through a single FP64 plan (vg_run_steps, with storage)."""
    from vlapy_gb300 import initializers as I
    from vlapy_gb300.plan import Plan, history_struct
    nx, nv, k = r["nx"], r["nv"], r["k"]
    dx, x, kx, inv = I.initialize_spatial_quantities(0.0, 2 * np.pi / k, nx)
    dv, v, kv = I.initialize_velocity_quantities(vmax, nv)
    p = Plan(nx, nv, x, v, kx, kv, inv, dx, dv, dt=dt, nu=r["nu"], collision="dg" if r["nu"] > 0 else "none")
    f = torch.as_tensor(I.initialize_distribution(nx, nv, vmax) * (1.0 + r["amplitude"] * np.cos(k * x))[:, None],
                        device="cuda")
    e = torch.zeros(nx, dtype=torch.float64, device="cuda")
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device="cuda")  # noqa: E731
    st = {"stored_f": torch.zeros((nsteps, 1, nv), dtype=torch.complex64, device="cuda"),
          "fields": {kk: z(nsteps, nx) for kk in vo.FIELD_KEYS},
          "series": {kk: z(nsteps) for kk in vo.SERIES_KEYS}}
    tb = torch.as_tensor(dt * np.arange(nsteps), device="cuda")
    p.run_steps(f, e, history_struct(st, nx, 1), tb, None, 0, nsteps, use_graph=False)
    return f, e, st


def test_batch_runs_equal_single_plans():
    """Each run of a batch of mixed shapes gives a single plan's f, e, field
    history and series bit for bit (the same device code per run)."""
    from vlapy_gb300.batch import Batch64
    runs = mixed_runs()
    b = Batch64(runs)
    f, e = b.initial_state()
    nsteps = 6
    eh, sh = b.history(nsteps)
    b.run_steps(f, e, nsteps, eh, sh)
    torch.cuda.synchronize()
    for i, r in enumerate(runs):
        pf, pe, st = _plan_steps(r, nsteps)
        assert torch.equal(b.f_of(f, i), pf), i
        assert torch.equal(b.e_of(e, i), pe), i
        assert torch.equal(b.e_of(eh, i), st["fields"]["e"]), i
        ser = b.series_of(sh, i)
        for q, kk in enumerate(vo.SERIES_KEYS):
            if kk == "mean_de2":
                continue
            assert torch.equal(ser[:, q], st["series"][kk]), (i, kk)


def test_batch_matches_oracle_and_graph():
    """Twenty steps against the oracle, and the graph replay equal to the
    direct launches."""
    from vlapy_gb300.batch import Batch64
    runs = [dict(nx=32, nv=256, k=0.31, amplitude=1e-2, nu=1e-3), dict(nx=64, nv=1024, k=0.4, amplitude=1e-3, nu=0.0),
            dict(nx=128, nv=512, k=0.27, amplitude=3e-3, nu=1e-2)]
    b = Batch64(runs)
    f1, e1 = b.initial_state()
    f2, e2 = f1.clone(), e1.clone()
    nsteps = 20
    b.run_steps(f1, e1, nsteps)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        b.run_steps(f2, e2, nsteps, use_graph=True, stream=s)
    torch.cuda.synchronize()
    assert torch.equal(f1, f2) and torch.equal(e1, e2)
    for i, r in enumerate(runs):
        nx, nv, k = r["nx"], r["nv"], r["k"]
        run = vo.OracleRun(nx, nv, 2 * np.pi / k, 6.4, 0.1, nu=r["nu"], operator="dg")
        dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
        fo = vo.maxwellian(nx, nv, 6.4) * (1.0 + r["amplitude"] * np.cos(k * x))[:, None]
        eo = np.zeros(nx)
        for it in range(nsteps):
            eo, fo = run.step(eo, fo, 0.1 * it)
        assert rel(b.f_of(f1, i).cpu().numpy(), fo) <= TOL * nsteps
        assert rel(b.e_of(e1, i).cpu().numpy(), eo) <= TOL * nsteps


def test_batch_landau_golden():
    """The reference's own Landau steps (fixture landau_32x512: 32 x 512,
    k = 0.3, A = 1e-4, 10 steps) as a batch of one run next to two others."""
    from vlapy_gb300.batch import Batch64
    d = np.load(os.path.join(G, "landau_32x512.npz"))
    runs = [dict(nx=64, nv=256, k=0.35, amplitude=1e-3, nu=1e-3), dict(nx=32, nv=512, k=0.3, amplitude=1e-4, nu=0.0),
            dict(nx=32, nv=512, k=0.4, amplitude=1e-2, nu=1e-4)]
    b = Batch64(runs)
    f, e = b.initial_state()
    # the fixture's own f0 (host libm exp/cos may differ in the last bit
    # between machines; the state is the reference's)
    np.testing.assert_allclose(b.f_of(f, 1).cpu().numpy(), d["f0"], rtol=1e-15, atol=0)
    b.f_of(f, 1).copy_(torch.as_tensor(d["f0"], device="cuda"))
    eh, sh = b.history(10)
    b.run_steps(f, e, 10, eh, sh)
    torch.cuda.synchronize()
    assert rel(b.f_of(f, 1).cpu().numpy(), d["f_10"]) <= TOL * 10
    assert rel(b.e_of(e, 1).cpu().numpy(), d["e_10"]) <= TOL * 10
    assert rel(b.e_of(eh, 1).cpu().numpy(), d["fields_e"]) <= 1e-11
    ser = b.series_of(sh, 1).cpu().numpy()
    for q, kk in enumerate(vo.SERIES_KEYS):
        ref = d["series_" + kk]
        atol = 1e-14 if kk != "mean_j" else 1e-12 * vo.trapz(np.abs(d["f0"]) * np.abs(vo.velocity_axis(6.4, 512)[1]),
                                                              vo.velocity_axis(6.4, 512)[0], 1).mean()
        np.testing.assert_allclose(ser[:, q], ref, rtol=1e-11, atol=atol, err_msg=kk)


def test_batch_rejects_bad_layouts():
    from vlapy_gb300.batch import Batch64
    with pytest.raises(NotImplementedError):
        Batch64([dict(nx=12, nv=64, k=0.3, amplitude=1e-3, nu=0.0)])
    b = Batch64([dict(nx=8, nv=64, k=0.3, amplitude=1e-3, nu=0.0)])
    f, e = b.initial_state()
    with pytest.raises(ValueError):
        b.run_steps(f[:-1], e, 1)

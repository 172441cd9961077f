"""The alternative FP64 steppers on the GPU: semi-Lagrangian x and v steps and
the centred-difference v step (vlapy/core/vlasov.py:42-80, 143-210), through
libvlagpu.so against the oracle and the reference's golden vectors.

Bar: the centred difference is NumPy's arithmetic and is checked bit for bit;
the semi-Lagrangian steps solve the same not-a-knot cubic spline as the
reference's FITPACK call by a different elimination, and are checked to a
relative L2 of 1e-12 per step.
"""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import vlapy_oracle as vo  # noqa: E402

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")
TOL_SL = 1e-12


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module", autouse=True)
def _lib_loaded():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import _lib
    _lib.load()


def cuda(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def make_case(nx, nv, seed=0, precision="fp64"):
    from vlapy_gb300.plan import Plan
    k, vmax = 0.3, 6.4
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    dv, v, kv = vo.velocity_axis(vmax, nv)
    rng = np.random.default_rng(seed)
    f = vo.maxwellian(nx, nv, vmax) * (1.0 + 0.05 * np.cos(k * x))[:, None]
    f = f + 1e-3 * rng.standard_normal((nx, nv))
    e = 0.2 * np.sin(k * x) + 0.05
    fbg = f.mean(axis=0) if precision == "fp32-deltaf" else None
    p = Plan(nx, nv, x, v, kx, kv, inv, dx, dv, dt=0.1, precision=precision, f_background=fbg)
    return p, f, e, x, v, dv


# shapes include the smallest grids the reference accepts, odd and
# non-power-of-two sizes, and the single-run workload grids
CD2_SHAPES = [(16, 64), (7, 3), (5, 1000), (64, 1024), (3, 17), (32, 512)]
SL_SHAPES = [(16, 64), (4, 4), (12, 96), (33, 20), (64, 1024), (128, 256), (32, 512)]


@pytest.mark.parametrize("nx,nv", CD2_SHAPES)
def test_cd2_bit_exact_with_oracle(nx, nv):
    p, f, e, x, v, dv = make_case(nx, nv)
    fin = cuda(f)
    for dt in (0.1, -0.37):
        out = p.edfdv_cd2(fin, cuda(e), torch.empty_like(fin), dt)
        np.testing.assert_array_equal(out.cpu().numpy(), vo.edfdv_center_differenced(f, e, dv, dt))
    np.testing.assert_array_equal(fin.cpu().numpy(), f)


@pytest.mark.parametrize("nx,nv", SL_SHAPES)
def test_sl_matches_oracle(nx, nv):
    p, f, e, x, v, dv = make_case(nx, nv, seed=nx + nv)
    fin = cuda(f)
    # dt = 2.5 carries the outer departure points past the padded grid (clamped)
    for dt in (0.1, 2.5, -0.6):
        gx = p.vdfdx_sl(fin, torch.empty_like(fin), dt).cpu().numpy()
        assert rel(gx, vo.vdfdx_sl(f, x, v, dt)) <= TOL_SL
        gv = p.edfdv_sl(fin, cuda(e), torch.empty_like(fin), dt).cpu().numpy()
        assert rel(gv, vo.edfdv_sl(f, e, x, v, dt)) <= TOL_SL
    np.testing.assert_array_equal(fin.cpu().numpy(), f)


def test_sl_smallest_grids():
    """x step at nx = 3 (the padded x grid needs x[2]) and v step at nv = 3."""
    p, f, e, x, v, dv = make_case(3, 8)
    gx = p.vdfdx_sl(cuda(f), cuda(np.zeros_like(f)), 0.3).cpu().numpy()
    assert rel(gx, vo.vdfdx_sl(f, x, v, 0.3)) <= TOL_SL
    p, f, e, x, v, dv = make_case(8, 3)
    gv = p.edfdv_sl(cuda(f), cuda(e), cuda(np.zeros_like(f)), 0.3).cpu().numpy()
    assert rel(gv, vo.edfdv_sl(f, e, x, v, 0.3)) <= TOL_SL


@pytest.mark.parametrize("tag,dt", [("0p1", 0.1), ("2p5", 2.5)])
def test_alternatives_match_golden(tag, dt):
    d = np.load(os.path.join(G, "advect_alt_16x64.npz"))
    p, _, _, x, v, dv = make_case(16, 64)
    np.testing.assert_array_equal(x, d["x"])
    f, e = cuda(d["f"]), cuda(d["e"])
    out = torch.empty_like(f)
    assert rel(p.vdfdx_sl(f, out, dt).cpu().numpy(), d["vdfdx_sl_" + tag]) <= TOL_SL
    assert rel(p.edfdv_sl(f, e, out, dt).cpu().numpy(), d["edfdv_sl_" + tag]) <= TOL_SL
    np.testing.assert_array_equal(p.edfdv_cd2(f, e, out, dt).cpu().numpy(), d["edfdv_cd2_" + tag])


def test_sl_leapfrog_run_matches_oracle():
    """Ten steps of the composed leapfrog with both semi-Lagrangian steppers and
    Dougherty collisions, through the reference-shaped closures."""
    from vlapy_gb300.core import collisions, field, vlasov, vlasov_poisson
    nx, nv, k, vmax, dt, nu = 32, 128, 0.3, 6.4, 0.1, 1e-3
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    dv, v, kv = vo.velocity_axis(vmax, nv)
    f0 = vo.maxwellian(nx, nv, vmax) * (1.0 + 1e-2 * np.cos(k * x))[:, None]
    stuff = {"nx": nx, "nv": nv, "x": x, "v": v, "kx": kx, "kv": kv, "one_over_kx": inv, "dv": dv,
             "dt": dt, "nu": nu, "driver_function": None, "f": f0}
    params = {"nu": nu, "fokker-planck": {"type": "dg", "solver": "batched_tridiagonal"},
              "backend": {"core": "gb300", "precision": "fp64"}}
    vd = vlasov.get_vdfdx(stuff, "sl", params)
    ed = vlasov.get_edfdv(stuff, "sl", params)
    solver = field.get_field_solver(stuff, "spectral", params)
    vp = vlasov_poisson.get_time_integrator("leapfrog", vd, ed, solver, stuff)
    from vlapy_gb300.core.step import get_collision_step
    fp = get_collision_step(stuff, params)
    collisions.check_names(params["fokker-planck"])
    run = vo.OracleRun(nx, nv, 2 * np.pi / k, vmax, dt, nu=nu, operator="dg", vdfdx="sl", edfdv="sl")
    e_g, f_g = cuda(np.zeros(nx)), cuda(f0)
    e_o, f_o = np.zeros(nx), f0.copy()
    for i in range(10):
        e_g, f_g = vp(e=e_g, f=f_g, t=dt * i)
        f_g = fp(f=f_g)
        e_o, f_o = run.step(e_o, f_o, dt * i)
    assert rel(f_g.cpu().numpy(), f_o) <= 10 * TOL_SL
    assert rel(e_g.cpu().numpy(), e_o) <= 1e-10


def test_alternatives_reject_bad_calls():
    from vlapy_gb300.core import vlasov
    p, f, e, x, v, dv = make_case(16, 64)
    fin = cuda(f)
    with pytest.raises(ValueError):
        p.vdfdx_sl(fin, fin, 0.1)           # out of place only
    with pytest.raises(ValueError):
        p.edfdv_cd2(fin, cuda(e), fin, 0.1)
    p3, f3, e3, *_ = make_case(3, 64)
    with pytest.raises(ValueError):
        p3.edfdv_sl(cuda(f3), cuda(e3), cuda(np.zeros_like(f3)), 0.1)   # nx >= 4
    p4, f4, *_ = make_case(16, 3)
    with pytest.raises(ValueError):
        p4.vdfdx_sl(cuda(f4), cuda(np.zeros_like(f4)), 0.1)             # nv >= 4
    pf, ff, ef, *_ = make_case(16, 64, precision="fp32-deltaf")
    g = torch.zeros((16, 64), dtype=torch.float32, device="cuda")
    with pytest.raises(NotImplementedError):
        pf.vdfdx_sl(g, torch.empty_like(g), 0.1)
    stuff = {"nx": 16, "nv": 64, "x": x, "v": v, "dv": dv, "dt": 0.1, "f": f}
    with pytest.raises(NotImplementedError):
        vlasov.get_edfdv(stuff, "cd2", {"backend": {"precision": "fp32-deltaf"}})
    with pytest.raises(NotImplementedError):
        vlasov.get_vdfdx(stuff, "cd2")

"""The CPU oracle against golden vectors produced by the reference itself.

These run without a GPU.  They pin the oracle: the CUDA path is tested
against the oracle only because the oracle reproduces the reference's outputs
on the fixtures in tests/golden (made by tests/golden/make_golden.py).
"""

import os

import numpy as np
import pytest

from oracle import vlapy_oracle as vo

G = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return np.load(os.path.join(G, name + ".npz"))


def _run_fixture(d, driver=None):
    m = {k[5:]: d[k][()] for k in d.files if k.startswith("meta_")}
    nx, nv = int(m["nx"]), int(m["nv"])
    n_modes = None if int(m["n_modes"]) < 0 else int(m["n_modes"])
    run = vo.OracleRun(nx, nv, float(m["xmax"]), float(m["vmax"]), float(m["dt"]),
                       nu=float(m["nu"]), operator=str(m["fp_type"]),
                       integrator=str(m["time"]), driver=driver, n_modes=n_modes,
                       vdfdx=str(m.get("vdfdx", "exponential")), edfdv=str(m.get("edfdv", "exponential")))
    st = vo.new_storage(d["f0"], np.zeros(nx), int(m["nsteps"]), n_modes)
    st["time_batch"] = d["time"]
    st["driver_array_batch"] = d["driver_array"]
    snaps = {}
    for i in range(int(m["nsteps"])):
        st, _ = run.timestep(st, i)
        snaps[i + 1] = (st["f"].copy(), st["e"].copy())
    return run, st, snaps


def _pulse_driver(d, x):
    pulses = {"p": {k: float(d["pulse_" + k]) for k in ("k0", "w0", "a0", "t_L", "t_R", "t_wL", "t_wR")}}
    if "pulse_envelope" in d.files and str(d["pulse_envelope"]) == "sin2":
        p = pulses["p"]
        return lambda t: vo.driver_sin2(x, p["k0"], p["w0"], p["a0"], p["t_R"], t)
    return lambda t: vo.driver_tanh(x, pulses, t)


@pytest.mark.parametrize("name", ["landau_32x512", "driven_dg_16x256", "driven_lb_16x256",
                                  "integrator_pefrl_16x128", "integrator_h-sixth_16x128",
                                  "step_sl_dg_16x64", "step_cd2_16x64", "driven_sin2_dg_64x1024"])
def test_oracle_timestep_matches_reference(name):
    d = _load(name)
    driver = None
    if "pulse_k0" in d.files:
        _, x = vo.spatial_axis(0.0, float(d["meta_xmax"]), int(d["meta_nx"]))[:2]
        driver = _pulse_driver(d, x)
    run, st, snaps = _run_fixture(d, driver)
    for k in d.files:
        if k.startswith("f_") or k.startswith("e_"):
            step = int(k.split("_")[1])
            got = snaps[step][0 if k[0] == "f" else 1]
            np.testing.assert_array_equal(got, d[k], err_msg=k)
    # long runs keep every keep_every-th row of the fields (but e) and stored_f
    ke = int(d["meta_keep_every"]) if "meta_keep_every" in d.files else 1
    for k in vo.FIELD_KEYS:
        np.testing.assert_array_equal(st["fields"][k][::1 if k == "e" else ke], d["fields_" + k], err_msg=k)
    for k in vo.SERIES_KEYS:
        np.testing.assert_array_equal(st["series"][k], d["series_" + k], err_msg=k)
    np.testing.assert_array_equal(st["stored_f"][::ke], d["stored_f"])


@pytest.mark.parametrize("tag", ["0p1", "2p5"])
def test_oracle_alternative_steppers_match_reference(tag):
    """Semi-Lagrangian x and v steps and the centred-difference v step against
    the reference's own closures (vlapy/core/vlasov.py:42-80, 143-210)."""
    d = _load("advect_alt_16x64")
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / 0.3, 16)
    dv, v, kv = vo.velocity_axis(6.4, 64)
    np.testing.assert_array_equal(x, d["x"])
    np.testing.assert_array_equal(v, d["v"])
    dt = {"0p1": 0.1, "2p5": 2.5}[tag]
    f, e = d["f"], d["e"]
    np.testing.assert_array_equal(vo.vdfdx_sl(f, x, v, dt), d["vdfdx_sl_" + tag])
    np.testing.assert_array_equal(vo.edfdv_sl(f, e, x, v, dt), d["edfdv_sl_" + tag])
    np.testing.assert_array_equal(vo.edfdv_center_differenced(f, e, dv, dt), d["edfdv_cd2_" + tag])


@pytest.mark.parametrize("op", ["lb", "dg"])
@pytest.mark.parametrize("vs", [0.0, 0.5, 1.5])
def test_oracle_collisions_match_reference(op, vs):
    d = _load("collisions_2x1024")
    tag = "%s_vs%g" % (op, vs)
    nv, vmax = 1024, 6.0
    dv = 2 * vmax / nv
    v = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    fin = vo.shifted_maxwellian(2, v, 1.0, vs)
    np.testing.assert_array_equal(fin, d["fin_" + tag])
    g = fin.copy()
    for it in range(16):
        g = vo.collision_step(g, v, 1e-2, 0.1, dv, op)
        if it == 0:
            np.testing.assert_array_equal(g, d["f1_" + tag])
    np.testing.assert_array_equal(g, d["f16_" + tag])


def test_oracle_collision_conservation():
    """The reference's own conservation checks (tests/test_collisions.py:39-165)."""
    nv, vmax = 1024, 6.0
    dv = 2 * vmax / nv
    v = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    for op in ("lb", "dg"):
        f = vo.shifted_maxwellian(2, v, 1.0, 0.0)
        g = f.copy()
        for _ in range(16):
            g = vo.collision_step(g, v, 1e-2, 0.1, dv, op)
        np.testing.assert_almost_equal(f, g, decimal=4)
        f = vo.shifted_maxwellian(2, v, 1.0, 0.5)
        g = f.copy()
        for _ in range(16):
            g = vo.collision_step(g, v, 1e-2, 0.1, dv, op)
        np.testing.assert_almost_equal(vo.trapz(g, dv, 1), vo.trapz(f, dv, 1), decimal=4)
        np.testing.assert_almost_equal(vo.trapz(g * v ** 2, dv, 1), vo.trapz(f * v ** 2, dv, 1), decimal=4)


def test_oracle_poisson_matches_reference_and_analytic():
    d = _load("poisson_96")
    x, inv = d["x"], d["one_over_kx"]
    kp = 0.25
    analytic = [np.cos(kp * x) / kp, -np.sin(2 * kp * x) / 2.0 / kp,
                np.cos(2 * kp * x) / 2.0 / kp - np.sin(8 * kp * x) / 8.0 / kp]
    for i in range(3):
        got = vo.field_from_density(d["charge"][i], inv)
        np.testing.assert_array_equal(got, d["e"][i])
        np.testing.assert_almost_equal(got, analytic[i], decimal=4)


def test_oracle_dispersion_root_matches_table():
    d = _load("dispersion")
    for k0, wr, wi, r in zip(d["k0"], d["w_real_table"], d["w_imag_table"], d["root"]):
        got = vo.epw_root(float(k0))
        np.testing.assert_allclose(got, r, rtol=1e-12)
        np.testing.assert_almost_equal(got, wr + 1j * wi, decimal=4)


def test_trapz_is_numpy_pairwise_sum():
    """The FP64 GPU kernels reproduce np.trapezoid bit for bit by replaying
    NumPy's pairwise summation tree; pin that tree here on the host."""
    from vlapy_gb300 import pairwise
    rng = np.random.default_rng(3)
    for n in (2, 3, 9, 17, 128, 129, 130, 511, 512, 1024, 4097, 8192):
        y = rng.standard_normal(n) + 1.0
        assert pairwise.trapz_emulated(y, 0.0234375) == np.trapezoid(y, dx=0.0234375)

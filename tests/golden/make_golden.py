"""Generate golden input/output vectors by running the reference VlaPy itself.

Run in a container where the reference source tree is available:

    python tests/golden/make_golden.py REFERENCE_ROOT [advect_alt|driven_sin2]

The reference is pure Python; it is imported unmodified with two shims:
``np.trapz = np.trapezoid`` (NumPy 2 removed trapz) and a stub ``mlflow``
module (vlapy/initializers.py imports it at module level; nothing used here
logs).  Outputs are small ``.npz`` files next to this script.  GPU test runs
never read the reference tree; they read these fixtures.
"""

from __future__ import annotations

import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(root):
    np.trapz = np.trapezoid
    sys.modules.setdefault("mlflow", types.ModuleType("mlflow"))
    sys.path.insert(0, root)
    from vlapy import initializers, field_driver  # noqa: F401
    from vlapy.core import step, field, collisions, vlasov  # noqa: F401
    from vlapy.diagnostics import z_function  # noqa: F401
    from tests import helpers  # noqa: F401
    from tests.extras import canosa_values  # noqa: F401
    return types.SimpleNamespace(
        initializers=initializers, field_driver=field_driver, step=step,
        field=field, collisions=collisions, vlasov=vlasov,
        z_function=z_function, helpers=helpers, canosa=canosa_values)


def _stuff(ref, nx, nv, xmax, vmax, dt, nu, driver_function, n_modes):
    dx, x, kx, inv_kx = ref.initializers.initialize_spatial_quantities(0.0, xmax, nx)
    dv, v, kv = ref.initializers.initialize_velocity_quantities(vmax, nv)
    # the LandauDamping rule dict (vlapy/diagnostics/landau_damping.py:34-37); note the
    # reference slices len(rule_dict) modes (vlapy/core/step.py:130-135), which equals
    # len(space) only because this dict has exactly two keys
    rules = ({"time": "first-last", "space": "all"} if n_modes is None
             else {"time": "first-last", "space": ["k%d" % m for m in range(n_modes)]})
    return {
        "nx": nx, "nv": nv, "x": x, "v": v, "kx": kx, "kv": kv, "one_over_kx": inv_kx,
        "dv": dv, "dt": dt, "nu": nu, "driver_function": driver_function,
        "rules_to_store_f": rules,
    }


def _params(time="leapfrog", fp_type="dg", nu=0.0, vdfdx="exponential", edfdv="exponential"):
    return {
        "nu": nu,
        "fokker-planck": {"type": fp_type, "solver": "batched_tridiagonal"},
        "vlasov-poisson": {"time": time, "vdfdx": vdfdx,
                           "edfdv": edfdv, "poisson": "spectral"},
        "backend": {"core": "numpy"},
    }


def _sim_config(stuff, f, nt, n_modes):
    nx = f.shape[0]
    if n_modes is None:
        stored = np.zeros((nt, nx, f.shape[1]))
        stored[0] = f
    else:
        stored = np.zeros((nt, n_modes, f.shape[1]), dtype=np.complex64)
        stored[0] = np.fft.fft(f, axis=0)[:n_modes]
    series = ["mean_n", "mean_j", "mean_T", "mean_e2", "mean_de2", "mean_f2", "mean_flogf"]
    fields = ["e", "driver", "n", "j", "T", "q", "fv4", "vN"]
    return {
        "time_batch": np.zeros(nt), "e": np.zeros(nx), "f": f.copy(), "stored_f": stored,
        "mean_cum_de2_previous": 0.0,
        "series": {k: np.zeros(nt) for k in series},
        "fields": {k: np.zeros((nt, nx)) for k in fields},
    }


def run_steps(ref, name, nx, nv, xmax, vmax, dt, nu, f0, nsteps, time="leapfrog",
              fp_type="dg", pulses=None, n_modes=2, snapshots=(1,), vdfdx="exponential",
              edfdv="exponential", driver=None, keep_every=1):
    """Run get_timestep (vlapy/core/step.py:286-328) from f0, e=0 and save the
    storage arrays plus f/e after the listed step counts.  driver: a closure
    of x returning the driver function, in place of the reference's tanh
    pulses; keep_every > 1 keeps only every keep_every-th row of the stored
    fields (except e) and of stored_f, to keep a long run's fixture small."""
    dx, x, kx, inv_kx = ref.initializers.initialize_spatial_quantities(0.0, xmax, nx)
    if driver is not None:
        drv = driver(x)
    elif pulses is None:
        drv = lambda t: np.zeros(nx)  # noqa: E731
    else:
        drv = ref.field_driver.get_driver_function(x=x, pulse_dictionary=pulses, np=np)
    stuff = _stuff(ref, nx, nv, xmax, vmax, dt, nu, drv, n_modes)
    ts = ref.step.get_timestep(_params(time, fp_type, nu, vdfdx, edfdv), stuff)
    t = dt * np.arange(nsteps)
    driver_array = np.array([drv(tt) for tt in t])
    sc = _sim_config(stuff, f0, nsteps, n_modes)
    sc["time_batch"] = t
    sc["driver_array_batch"] = driver_array
    out = {"f0": f0, "time": t, "driver_array": driver_array}
    for i in range(nsteps):
        sc, _ = ts(sc, i)
        if (i + 1) in snapshots:
            out["f_%d" % (i + 1)] = np.array(sc["f"])
            out["e_%d" % (i + 1)] = np.array(sc["e"])
    for k, val in sc["fields"].items():
        out["fields_" + k] = val if k == "e" else val[::keep_every]
    for k, val in sc["series"].items():
        out["series_" + k] = val
    out["stored_f"] = sc["stored_f"][::keep_every]
    meta = dict(nx=nx, nv=nv, xmax=xmax, vmax=vmax, dt=dt, nu=nu, nsteps=nsteps,
                time=time, fp_type=fp_type, n_modes=-1 if n_modes is None else n_modes,
                vdfdx=vdfdx, edfdv=edfdv, keep_every=keep_every)
    for k, val in meta.items():
        out["meta_" + k] = np.array(val)
    if pulses is not None:
        p = list(pulses.values())[0]
        for k in ("k0", "w0", "a0", "t_L", "t_R", "t_wL", "t_wR"):
            out["pulse_" + k] = np.array(p[k])
        out["pulse_envelope"] = np.array(p.get("envelope", "tanh"))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, sorted(out.keys())[:6], "...")


def advect_alt(ref):
    """The alternative steppers of vlapy/core/vlasov.py: semi-Lagrangian in x
    and v (:42-80, :168-210) and the centred difference in v (:143-165), each
    called directly, plus short runs of the full timestep that use them."""
    I = ref.initializers
    k, nx, nv, vmax = 0.3, 16, 64, 6.4
    dx, x, kx, inv_kx = I.initialize_spatial_quantities(0.0, 2 * np.pi / k, nx)
    dv, v, kv = I.initialize_velocity_quantities(vmax, nv)
    rng = np.random.default_rng(11)
    f = I.initialize_distribution(nx, nv, vmax) * (1.0 + 0.05 * np.cos(k * x))[:, None]
    f = f + 1e-3 * rng.standard_normal((nx, nv))
    e = 0.2 * np.sin(k * x) + 0.05
    out = {"x": x, "v": v, "dv": np.array(dv), "f": f, "e": e}
    vd_sl = ref.vlasov.get_vdfdx_sl(x=x, v=v)
    ed_sl = ref.vlasov.get_edfdv_sl(x=x, v=v)
    ed_cd2 = ref.vlasov.get_edfdv_center_differenced(dv=dv)
    # dt = 2.5 moves the outer departure points past the padded grid (clamped)
    for tag, dt in (("0p1", 0.1), ("2p5", 2.5)):
        out["vdfdx_sl_" + tag] = vd_sl(f, dt)
        out["edfdv_sl_" + tag] = ed_sl(f, e, dt)
        out["edfdv_cd2_" + tag] = ed_cd2(f, e, dt)
    np.savez_compressed(os.path.join(HERE, "advect_alt_16x64.npz"), **out)
    print("wrote advect_alt_16x64")

    f0 = I.initialize_distribution(nx, nv, vmax) * (1.0 + 1e-2 * np.cos(k * x))[:, None]
    run_steps(ref, "step_sl_dg_16x64", nx, nv, 2 * np.pi / k, vmax, 0.1, 1e-3, f0, 3,
              fp_type="dg", snapshots=(1, 3), vdfdx="sl", edfdv="sl")
    run_steps(ref, "step_cd2_16x64", nx, nv, 2 * np.pi / k, vmax, 0.1, 0.0, f0, 3,
              snapshots=(1, 3), edfdv="cd2")


def driven_sin2(ref):
    """The driven electron-plasma-wave workload on its own grid: 64 x 1024,
    k = 0.3, vmax = 6.4, Maxwellian start, Dougherty collisions nu = 1e-3,
    dt = 0.1, and the external field a0 sin(k x - w t) sin^2(pi t / 100) on
    [0, 100] (zero after), a0 = 1e-2, w the real part of the reference's
    dispersion root.  The reference has no such envelope; its step calls any
    driver closure (vlapy/core/vlasov_poisson.py:55), so the closure is
    written here.  150 steps (t up to 15, the envelope rising); f at the
    last step, e at every step, the other fields and stored_f every 10th."""
    I = ref.initializers
    k, nx, nv, vmax, a0, t_end = 0.3, 64, 1024, 6.4, 1e-2, 100.0
    w = float(np.real(ref.z_function.get_roots_to_electrostatic_dispersion(1.0, 1.0, k)))

    def closure(x):
        def drv(t):
            if t < 0.0 or t > t_end:
                return np.zeros(x.size)
            s = math.sin(math.pi * t / t_end)
            return (a0 * (s * s)) * np.sin(k * x - w * t)
        return drv

    pulses = {"p": {"k0": k, "w0": w, "a0": a0, "t_L": 0.0, "t_R": t_end, "t_wL": 1.0, "t_wR": 1.0,
                    "envelope": "sin2"}}
    f0 = I.initialize_distribution(nx, nv, vmax)
    run_steps(ref, "driven_sin2_dg_64x1024", nx, nv, 2 * np.pi / k, vmax, 0.1, 1e-3, f0, 150,
              fp_type="dg", pulses=pulses, snapshots=(150,), driver=closure, keep_every=10)


def main(root):
    ref = _import_reference(root)
    I = ref.initializers

    # 1. Landau damping, leapfrog, no collisions: 32x512, k=0.3, vmax=6.4,
    #    A=1e-4, dt=0.1 (the plain Landau workload's grid; tests/test_landau_damping.py:53-79
    #    use the same default grid).
    k = 0.3
    nx, nv, vmax = 32, 512, 6.4
    dx, x, kx, inv_kx = I.initialize_spatial_quantities(0.0, 2 * np.pi / k, nx)
    f0 = I.initialize_distribution(nx, nv, vmax) * (1.0 + 1e-4 * np.cos(k * x))[:, None]
    run_steps(ref, "landau_32x512", nx, nv, 2 * np.pi / k, vmax, 0.1, 0.0, f0, 10,
              snapshots=(1, 2, 10))

    # 2. Driven wave with Dougherty collisions and the reference tanh pulse
    #    (vlapy/field_driver.py:24-50): 16x256, nu=1e-3.
    nx, nv = 16, 256
    root_w = ref.z_function.get_roots_to_electrostatic_dispersion(1.0, 1.0, k)
    pulses = {"p": {"k0": k, "w0": float(np.real(root_w)), "a0": 1e-2, "t_L": 0.2,
                    "t_R": 5.0, "t_wL": 0.5, "t_wR": 0.5}}
    dx, x, kx, inv_kx = I.initialize_spatial_quantities(0.0, 2 * np.pi / k, nx)
    f0 = I.initialize_distribution(nx, nv, vmax) * (1.0 + 1e-3 * np.cos(k * x))[:, None]
    run_steps(ref, "driven_dg_16x256", nx, nv, 2 * np.pi / k, vmax, 0.1, 1e-3, f0, 6,
              fp_type="dg", pulses=pulses, snapshots=(1, 6))
    run_steps(ref, "driven_lb_16x256", nx, nv, 2 * np.pi / k, vmax, 0.1, 1e-2, f0, 3,
              fp_type="lb", pulses=pulses, snapshots=(1, 3))

    # 3. Higher-order integrators on a small grid, store-all rule.
    nx, nv = 16, 128
    dx, x, kx, inv_kx = I.initialize_spatial_quantities(0.0, 2 * np.pi / k, nx)
    f0 = I.initialize_distribution(nx, nv, vmax) * (1.0 + 1e-2 * np.cos(k * x))[:, None]
    for integ in ("pefrl", "h-sixth"):
        run_steps(ref, "integrator_%s_16x128" % integ, nx, nv, 2 * np.pi / k, vmax, 0.1, 0.0,
                  f0, 3, time=integ, n_modes=None, snapshots=(1, 3))

    # 4. Collision-operator fixtures: tests/test_collisions.py:168-211
    #    (nx=2, nv=1024, nu=1e-2, dt=0.1, vmax=6, 16 steps).
    out = {}
    nvc, vmaxc = 1024, 6.0
    dvc = 2 * vmaxc / nvc
    vc = np.linspace(-vmaxc + dvc / 2.0, vmaxc - dvc / 2.0, nvc)
    for op in ("lb", "dg"):
        for vs in (0.0, 0.5, 1.5):
            fin = ref.helpers.__initialize_f__(nx=2, v=vc, v0=1.0, vshift=vs)
            stuff = {"f": fin, "v": vc, "nv": nvc, "nx": 2, "nu": 1e-2, "dt": 0.1, "dv": dvc}
            params = {"fokker-planck": {"type": op, "solver": "batched_tridiagonal"}, "nu": 1e-2}
            fp = ref.step.get_collision_step(all_params=params, stuff_for_time_loop=stuff)
            g = fin.copy()
            tag = "%s_vs%g" % (op, vs)
            out["fin_" + tag] = fin
            for it in range(16):
                g = fp(g)
                if it == 0:
                    out["f1_" + tag] = g.copy()
            out["f16_" + tag] = g
    np.savez_compressed(os.path.join(HERE, "collisions_2x1024.npz"), **out)
    print("wrote collisions_2x1024")

    # 5. Spectral Poisson against analytic fields: tests/test_fieldsolver.py:27-53 (nx=96).
    nxp, kp = 96, 0.25
    xm = 2 * np.pi / kp
    dxp = xm / nxp
    ax = np.linspace(dxp / 2, xm - dxp / 2, nxp)
    kxp = np.fft.fftfreq(ax.size, d=dxp) * 2.0 * np.pi
    inv = np.zeros_like(kxp)
    inv[1:] = 1.0 / kxp[1:]
    rho = np.stack([1.0 + np.sin(kp * ax), 1.0 + np.cos(2 * kp * ax),
                    1.0 + np.sin(2 * kp * ax) + np.cos(8 * kp * ax)])
    e_ref = np.stack([ref.field.solve_for_field(charge_density=1.0 - r, one_over_kx=inv) for r in rho])
    np.savez_compressed(os.path.join(HERE, "poisson_96.npz"), x=ax, one_over_kx=inv,
                        charge=1.0 - rho, e=e_ref)
    print("wrote poisson_96")

    # 6. Dispersion roots: the reference's known-answer table
    #    (tests/test_zsolver.py:7-15, tests/extras/canosa_values.py) and its solver.
    k0s = np.array(ref.canosa.k0)
    roots = np.array([ref.z_function.get_roots_to_electrostatic_dispersion(1.0, 1.0, kk) for kk in k0s])
    np.savez_compressed(os.path.join(HERE, "dispersion.npz"), k0=k0s,
                        w_real_table=np.array(ref.canosa.w_real),
                        w_imag_table=np.array(ref.canosa.w_imag), root=roots)
    print("wrote dispersion")

    advect_alt(ref)
    driven_sin2(ref)


if __name__ == "__main__":
    # `make_golden.py ROOT` writes every fixture; `make_golden.py ROOT advect_alt`
    # (or `driven_sin2`) writes only those of the alternative steppers (or of
    # the sin^2-driven wave)
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py REFERENCE_ROOT [advect_alt|driven_sin2]")
    root = sys.argv[1]
    if len(sys.argv) > 2 and sys.argv[2] == "advect_alt":
        advect_alt(_import_reference(root))
    elif len(sys.argv) > 2 and sys.argv[2] == "driven_sin2":
        driven_sin2(_import_reference(root))
    else:
        main(root)

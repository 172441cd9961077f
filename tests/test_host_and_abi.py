"""CPU-only checks: the C-ABI library builds, loads and exports every symbol
of include/vlagpu.h; host-side logic (rule handling, name validation, the
NumPy summation tree) behaves like the reference.  No compute call is made."""

import ctypes
import os
import re
import shutil

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "vlagpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(vg_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from vlapy_gb300 import build
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        if not os.path.exists(build.LIB):
            pytest.skip("no nvcc and no prebuilt library")
        return build.LIB
    return build.build()


def test_header_declares_the_abi():
    fns = header_functions()
    for name in ("vg_plan_create", "vg_plan_destroy", "vg_last_error", "vg_edfdv", "vg_vdfdx",
                 "vg_charge_density", "vg_poisson", "vg_field_solve", "vg_collision_step",
                 "vg_storage_step", "vg_driver", "vg_run_steps"):
        assert name in fns


def test_library_exports_every_header_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.vg_version() >= 1


C_CONSUMER = r"""
#include <stdio.h>
#include "vlagpu.h"
int main(void) {
  vg_plan* p = 0;
  int v = vg_version();
  int st = vg_plan_create(NULL, &p);
  printf("%d %d %s\n", v, st, vg_last_error());
  return (v >= 1 && st == VG_ERR_ARG && p == NULL) ? 0 : 1;
}
"""


@pytest.mark.parametrize("compiler,std", [("gcc", "-std=c99"), ("g++", "-std=c++17")])
def test_header_serves_a_c_consumer(lib_path, tmp_path, compiler, std):
    """What a cgo / JNI / plain C binding does first: compile against the header
    with warnings as errors, link libvlagpu.so, and make the calls that need no
    GPU (the version, and a plan refused for a null descriptor)."""
    import subprocess
    if shutil.which(compiler) is None:
        pytest.skip(compiler + " not installed")
    src = tmp_path / ("consumer.c" if compiler == "gcc" else "consumer.cpp")
    src.write_text(C_CONSUMER)
    exe = str(tmp_path / "consumer")
    libdir = os.path.dirname(lib_path)
    cmd = [compiler, std, "-Wall", "-Wextra", "-Werror", "-pedantic", str(src), "-I",
           os.path.join(ROOT, "include"), "-L", libdir, "-lvlagpu", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "null descriptor" in r.stdout


def test_binding_covers_header(lib_path):
    from vlapy_gb300 import _lib
    assert set(header_functions()) <= set(_lib.EXPORTS)


def test_plan_create_rejects_bad_descriptor(lib_path):
    """Argument checks run before any CUDA call."""
    from vlapy_gb300 import _lib
    lib = _lib.load(lib_path)
    d = _lib.VgRunDesc()
    d.nx, d.nv = 1, 8
    h = ctypes.c_void_p()
    assert lib.vg_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.VG_ERR_ARG
    assert b"nx and nv" in lib.vg_last_error()
    assert lib.vg_plan_create(None, ctypes.byref(h)) == _lib.VG_ERR_ARG
    assert lib.vg_edfdv(None, None, None, 0.1, None) == _lib.VG_ERR_ARG


def test_sweep_create_rejects_bad_runs(lib_path):
    """The sweep's argument checks run before any CUDA call: no runs, a bad
    descriptor, and runs outside the supported shape classes (the error names
    the run)."""
    from vlapy_gb300 import _lib
    lib = _lib.load(lib_path)
    h = ctypes.c_void_p()

    def create(runs, n=None, collision=_lib.VG_COLL_DG, vmax=6.4):
        arr = (_lib.VgSweepRun * max(1, len(runs)))(*[_lib.VgSweepRun(*r) for r in runs])
        d = _lib.VgSweepDesc(len(runs) if n is None else n, collision, vmax, 0.1, arr)
        return lib.vg_sweep_create(ctypes.byref(d), ctypes.byref(h))

    ok = (32, 256, 0.3, 1e-3, 1e-3)
    assert create([], n=0) == _lib.VG_ERR_ARG
    assert create([ok], vmax=0.0) == _lib.VG_ERR_ARG
    assert create([ok], collision=_lib.VG_COLL_NONE) == _lib.VG_ERR_ARG
    assert lib.vg_sweep_create(None, ctypes.byref(h)) == _lib.VG_ERR_ARG
    for bad in ((12, 256, 0.3, 1e-3, 1e-3),    # nx not a power of two
                (512, 256, 0.3, 1e-3, 1e-3),   # nx above 256
                (32, 96, 0.3, 1e-3, 1e-3),     # nv not a power of two
                (32, 4096, 0.3, 1e-3, 1e-3),   # nv above 2048
                (8, 256, 0.3, 1e-3, 1e-3),     # nv below the column tile width 4096 / nx
                (32, 256, 0.0, 1e-3, 1e-3),    # k = 0
                (32, 256, 0.3, 1e-3, -1e-3)):  # nu < 0
        assert create([ok, bad]) == _lib.VG_ERR_UNSUPPORTED, bad
        assert b"sweep run 1" in lib.vg_last_error()
    assert not h.value


def test_batch_create_rejects_bad_runs(lib_path):
    """The FP64 batch's argument checks run before any CUDA call."""
    from vlapy_gb300 import _lib
    lib = _lib.load(lib_path)
    h = ctypes.c_void_p()
    grid = (ctypes.c_double * 64)()

    def desc(nx=16, nv=32, precision=_lib.VG_F64, dt=0.1, nu=0.0, grids=True):
        d = _lib.VgRunDesc()
        d.nx, d.nv, d.precision, d.dt, d.nu = nx, nv, precision, dt, nu
        d.collision, d.integrator = _lib.VG_COLL_NONE, _lib.VG_LEAPFROG
        if grids:
            for name in ("x", "v", "kx", "kv", "one_over_kx", "v_pow"):
                setattr(d, name, grid)
        return d

    def create(*descs, n=None):
        arr = (_lib.VgRunDesc * max(1, len(descs)))(*descs)
        return lib.vg_batch_create(arr, len(descs) if n is None else n, ctypes.byref(h))

    assert create(n=0) == _lib.VG_ERR_ARG
    assert lib.vg_batch_create(None, 1, ctypes.byref(h)) == _lib.VG_ERR_ARG
    for bad, status in ((desc(precision=_lib.VG_F32_DELTA_F), _lib.VG_ERR_UNSUPPORTED),
                        (desc(nx=12), _lib.VG_ERR_UNSUPPORTED),
                        (desc(nx=2048), _lib.VG_ERR_UNSUPPORTED),
                        (desc(nv=16384), _lib.VG_ERR_UNSUPPORTED),
                        (desc(grids=False), _lib.VG_ERR_ARG),
                        (desc(dt=0.05), _lib.VG_ERR_ARG),
                        (desc(nu=-1e-3), _lib.VG_ERR_ARG)):
        assert create(desc(), bad) == status
        assert b"batch run 1" in lib.vg_last_error()
    assert not h.value


def test_struct_layout_matches_header(lib_path):
    from vlapy_gb300 import _lib
    names = ["vg_run_desc", "vg_history", "vg_pulse", "vg_sweep_run", "vg_sweep_desc", "vg_prof_entry",
             "vg_corr_batch"]
    src = ("#include <stdio.h>\n#include \"vlagpu.h\"\nint main(){"
           + "".join('printf("%%zu ", sizeof(%s));' % n for n in names) + "}")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(td, "s")
        subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    assert [int(x) for x in out] == [ctypes.sizeof(t) for t in (
        _lib.VgRunDesc, _lib.VgHistory, _lib.VgPulse, _lib.VgSweepRun, _lib.VgSweepDesc, _lib.VgProfEntry,
        _lib.VgCorrBatch)]


def test_pairwise_tables():
    from vlapy_gb300 import pairwise
    for n in (1, 7, 8, 127, 128, 129, 511, 1023, 8191):
        leaves, prog = pairwise.leaf_program(n)
        assert sum(ln for _, ln in leaves) == n
        assert all(ln <= 128 for _, ln in leaves)
        assert prog.count(-1) == len(leaves) - 1


def test_mode_count_follows_reference_rule_dict():
    from vlapy_gb300.core.step import n_modes_of
    assert n_modes_of({"time": "first-last", "space": ["k0", "k1"]}) == 2
    # the reference slices len(rule_dict) modes: one key -> one mode, broadcast
    assert n_modes_of({"space": ["k0", "k1"]}) == 1
    assert n_modes_of({"space": "all"}) is None
    with pytest.raises(NotImplementedError):
        n_modes_of({"space": ["x"]})


def test_stepper_arguments_checked_on_host():
    """The out-of-place steppers refuse a wrong dtype or shape before any pointer
    reaches a kernel."""
    import torch
    from vlapy_gb300.plan import check_f64
    t = torch.zeros((4, 8), dtype=torch.float64)
    assert check_f64(t, (4, 8), "f") is t
    with pytest.raises(ValueError):
        check_f64(t.float(), (4, 8), "f")
    with pytest.raises(ValueError):
        check_f64(t, (4, 9), "f")
    with pytest.raises(ValueError):
        check_f64(torch.zeros(5, dtype=torch.float64), (4,), "e")
    with pytest.raises(TypeError):
        check_f64(np.zeros((4, 8)), (4, 8), "f")


@pytest.mark.parametrize("name", ["leapfrog", "pefrl", "h-sixth"])
def test_composed_integrators_follow_the_oracle(name, monkeypatch):
    """The composed integrators of vlapy_gb300.core.vlasov_poisson (used with the
    semi-Lagrangian and centred-difference steppers, and with a Python driver
    closure) call the sub-operators in the reference's order with the
    reference's sub-step sizes and driver times.  Fed the oracle's NumPy
    closures they reproduce the oracle's integrators bit for bit."""
    from oracle import vlapy_oracle as vo
    from vlapy_gb300.core import vlasov_poisson as vp
    monkeypatch.setattr(vp, "as_device", np.asarray)  # host arrays stand in for device buffers
    k, nx, nv, dt, t = 0.3, 16, 64, 0.1, 1.7
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    dv, v, kv = vo.velocity_axis(6.4, nv)
    pulses = {"p": {"k0": k, "w0": 1.16, "a0": 1e-2, "t_L": 0.5, "t_R": 5.0, "t_wL": 0.5, "t_wR": 0.5}}

    def drv(tt):
        return vo.driver_tanh(x, pulses, tt)

    ops = vo.Operators(x, v, kx, kv, inv, dv, drv, vdfdx="sl", edfdv="cd2")
    step = vp.get_time_integrator(
        name, lambda f, dt: ops.vdfdx(f, dt), lambda f, e, dt: ops.edfdv(f, e, dt),
        lambda driver_field, f: vo.total_field(driver_field, f, dv, inv),
        {"dt": dt, "driver_function": drv, "nx": nx})
    f0 = vo.maxwellian(nx, nv, 6.4) * (1.0 + 1e-2 * np.cos(k * x))[:, None]
    e0 = 1e-3 * np.sin(k * x)
    e1, f1 = step(e=e0, f=f0, t=t)
    e2, f2 = vo.INTEGRATORS[name](ops, e0, f0, t, dt)
    np.testing.assert_array_equal(f1, f2)
    np.testing.assert_array_equal(e1, e2)


def test_unknown_names_raise_not_implemented():
    from vlapy_gb300.core import collisions
    with pytest.raises(NotImplementedError):
        collisions.check_names({"type": "bgk", "solver": "batched_tridiagonal"})
    with pytest.raises(NotImplementedError):
        collisions.check_names({"type": "dg", "solver": "lu"})
    assert collisions.check_names({"type": "dg", "solver": "naive"}) == ("dg", "naive")
    # stepper names are checked before any device plan is built: "cd2" exists
    # only for e df/dv, and the alternatives run in the fp64 mode only
    from vlapy_gb300.core import vlasov
    stuff = {"nx": 8, "nv": 16, "dv": 0.8, "dt": 0.1}
    with pytest.raises(NotImplementedError):
        vlasov.get_vdfdx(stuff, "cd2")
    with pytest.raises(NotImplementedError):
        vlasov.get_edfdv(stuff, "upwind")
    for name in ("sl", "cd2"):
        with pytest.raises(NotImplementedError):
            vlasov.get_edfdv(stuff, name, {"backend": {"precision": "fp32-deltaf"}})
    with pytest.raises(NotImplementedError):
        vlasov.get_vdfdx(stuff, "sl", {"backend": {"precision": "fp32-deltaf"}})


def test_host_driver_matches_oracle():
    from oracle import vlapy_oracle as vo
    from vlapy_gb300 import field_driver
    x = np.linspace(0.1, 20.0, 64)
    pulses = {"p": {"k0": 0.3, "w0": 1.16, "a0": 1e-2, "t_L": 6, "t_R": 20, "t_wL": 2.5, "t_wR": 2.5}}
    d = field_driver.get_driver_function(x, pulses)
    for t in (0.0, 6.0, 13.3, 40.0):
        np.testing.assert_array_equal(d(t), vo.driver_tanh(x, pulses, t))
    s2 = field_driver.get_driver_function(x, {"p": {"k0": 0.3, "w0": 1.16, "a0": 1e-2, "t_R": 100.0,
                                                    "envelope": "sin2"}})
    for t in (0.0, 33.0, 100.0, 120.0):
        np.testing.assert_array_equal(s2(t), vo.driver_sin2(x, 0.3, 1.16, 1e-2, 100.0, t))


def test_initializers_match_oracle():
    from oracle import vlapy_oracle as vo
    from vlapy_gb300 import initializers as I
    np.testing.assert_array_equal(I.initialize_distribution(8, 64, 6.4), vo.maxwellian(8, 64, 6.4))
    for a, b in zip(I.initialize_velocity_quantities(6.4, 64), vo.velocity_axis(6.4, 64)):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(I.initialize_spatial_quantities(0.0, 20.0, 32), vo.spatial_axis(0.0, 20.0, 32)):
        np.testing.assert_array_equal(a, b)
    p = I.specify_epw_params_to_dict(0.3, I.make_default_params_dictionary())
    np.testing.assert_allclose(p["w_epw"] + 1j * p["nu_ld"], vo.epw_root(0.3), rtol=1e-12)


def test_dispersion_root_matches_reference_roots():
    """The Newton root of the set-up module against the roots the reference's
    own solver wrote (vlapy/diagnostics/z_function.py:26-50, fixture
    dispersion.npz) and the Canosa table of tests/test_zsolver.py."""
    import os
    from oracle import vlapy_oracle as vo
    from vlapy_gb300 import dispersion
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "dispersion.npz"))
    for k0, wr, wi, r in zip(d["k0"], d["w_real_table"], d["w_imag_table"], d["root"]):
        got = dispersion.get_roots_to_electrostatic_dispersion(1.0, 1.0, float(k0))
        # the reference's secant iteration stops at a 1.5e-8 tolerance
        np.testing.assert_allclose(got, r, rtol=1e-8)
        np.testing.assert_almost_equal(got, wr + 1j * wi, decimal=4)
    # another starting frequency converges to the same root
    g = dispersion.get_roots_to_electrostatic_dispersion(1.0, 1.0, 0.3, initial_root_guess=1.1)
    np.testing.assert_allclose(g, vo.epw_root(0.3), rtol=1e-8)


def test_corrector_layout_and_restriction():
    """Corrector parameter layout (header, module, oracle agree) and the
    spectral restriction fine -> coarse velocity grid."""
    import re
    from oracle import corrector_oracle as co
    from vlapy_gb300 import corrector as cm
    from vlapy_gb300.initializers import initialize_distribution
    hdr = open(os.path.join(ROOT, "include", "vlagpu.h")).read()
    assert int(re.search(r"vg_corr_num_params\(\) =\s*\*?\s*(\d+)\s*\*?\s*floats", hdr).group(1)) == co.N_PARAMS
    assert cm.SHAPES == co.SHAPES
    p = cm.init_params(0)
    assert p.size == co.N_PARAMS and p.dtype == np.float32
    d = co.unpack(p)
    assert float(d["W4"].abs().max()) == 0.0 and float(d["b4"].abs().max()) == 0.0
    assert float(d["W1"][:, 4:].abs().max()) == 0.0
    np.testing.assert_array_equal(co.pack(d), p)
    # restriction: exact on what the coarse grid represents, and maps the
    # fine Maxwellian onto the coarse one
    R = cm.restriction_matrix(1024, 128)
    vf = -6.4 + 12.8 / 1024 * (np.arange(1024) + 0.5)
    vc = -6.4 + 12.8 / 128 * (np.arange(128) + 0.5)
    for m in (0, 1, 5, 63):
        kv = 2 * np.pi * m / 12.8
        np.testing.assert_allclose(R @ np.cos(kv * vf + 0.3), np.cos(kv * vc + 0.3), atol=1e-12)
    mf = initialize_distribution(1, 1024, 6.4)[0]
    mc = initialize_distribution(1, 128, 6.4)[0]
    assert np.abs(R @ mf - mc).max() < 1e-9
    # the collision-rate feature: zero without collisions, about 1 at nu = 1e-2
    f = cm.nu_feature([0.0, 1e-5, 1e-2])
    assert f[0] == 0.0 and 0.09 < f[1] < 0.11 and 0.99 < f[2] < 1.01


def test_corrector_oracle_emulation_close_to_fp64():
    """The BF16-emulating oracle differs from the FP64 network by BF16 noise only."""
    torch = pytest.importorskip("torch")
    from oracle import corrector_oracle as co
    from vlapy_gb300 import corrector as cm
    rng = np.random.default_rng(3)
    p = cm.init_params(1)
    d = co.unpack(p)
    d["W4"][:] = torch.as_tensor(rng.uniform(-0.1, 0.1, (1, 64, 5)))
    p = co.pack(d)
    g = rng.standard_normal((20, 128)).astype(np.float32)
    t = (g + 0.01 * rng.standard_normal((20, 128))).astype(np.float32)
    feat = np.full(20, 0.5, np.float32)
    le, ge = co.loss_and_grads(p, g, feat, t, 6.4, 0.01, emulate=True)
    lx, gx = co.loss_and_grads(p, g, feat, t, 6.4, 0.01, emulate=False)
    assert abs(le - lx) < 1e-3 * lx
    # BF16 operands in the forward pass move the early-layer gradients by a
    # few per cent on random data (sums with heavy cancellation)
    assert np.linalg.norm(ge - gx) < 0.15 * np.linalg.norm(gx)


def test_damping_fit_matches_oracle_fit():
    """The product's damping diagnostic and the oracle's fit agree on a
    synthetic damped standing wave and on an oracle Landau run."""
    from oracle import vlapy_oracle as vo
    from vlapy_gb300.diagnostics import damping_fit, mode_amplitude
    t = 0.1 * np.arange(1, 1201)
    amp = np.abs(np.exp(-0.0153 * t) * np.cos(1.41 * t + 0.2))
    r, w = damping_fit(t, amp, t_min=5.0)
    assert abs(r + 0.0153) < 1e-4 and abs(w - 1.41) < 1e-3
    assert (r, w) == pytest.approx(vo.envelope_fit(t, amp, t_min=5.0), rel=1e-12)
    e = np.random.default_rng(0).standard_normal((50, 16))
    np.testing.assert_array_equal(mode_amplitude(e), vo.mode_amplitude(e))
    assert np.isnan(damping_fit(t[:20], amp[:20])[0])


@pytest.mark.parametrize("rules", [{"time": "first-last", "space": ["k0", "k1"]},
                                   {"time": "all", "space": "all"}])
def test_storage_batch_layout_matches_reference(rules):
    """The sim_config layout of this backend goes through the conversion of
    StorageManager.batch_update (vlapy/storage.py:177-315): host arrays with
    the reference's keys, shapes and dtypes (the oracle's restatement of
    vlapy/outer_loop.py:149-215), each fitting the coordinates batch_update
    attaches.  Built in host memory here; the GPU tests run the same check on
    a sim_config that the inner loop has filled."""
    import torch
    from oracle import vlapy_oracle as vo
    from vlapy_gb300 import initializers as I, outer_loop, storage
    nx, nv, nt = 16, 64, 5
    dx, x, kx, inv = I.initialize_spatial_quantities(0.0, 2 * np.pi / 0.3, nx)
    dv, v, kv = I.initialize_velocity_quantities(6.4, nv)
    f = I.initialize_distribution(nx, nv, 6.4)
    stuff = {"f": f, "e": np.zeros(nx)}
    sc = outer_loop.get_arrays_for_inner_loop(stuff, nt, rules, device="cpu")
    sc["time_batch"] = torch.as_tensor(0.1 * np.arange(nt))
    sc["series"]["mean_de2"] += 1e-3
    sc = outer_loop.post_inner_loop_update(sc)
    ref = vo.new_storage(f, np.zeros(nx), nt, None if rules["space"] == "all" else len(rules["space"]))
    fields, stored_f, t, series, cur = storage.check_batch(sc, x, v, rules)
    assert set(fields) == set(ref["fields"]) and set(series) >= set(ref["series"])
    for k in ref["fields"]:
        assert fields[k].shape == ref["fields"][k].shape and fields[k].dtype == ref["fields"][k].dtype
    for k in ref["series"]:
        assert series[k].shape == ref["series"][k].shape and series[k].dtype == ref["series"][k].dtype
    assert stored_f.shape == ref["stored_f"].shape and stored_f.dtype == ref["stored_f"].dtype
    np.testing.assert_allclose(stored_f[0], ref["stored_f"][0], rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(cur, f)
    np.testing.assert_array_equal(t, 0.1 * np.arange(nt))
    # the post-batch series of vlapy/outer_loop.py:218-245
    np.testing.assert_allclose(series["mean_cum_de2"], 1e-3 * np.arange(1, nt + 1))
    assert sc["mean_cum_de2_previous"] == pytest.approx(1e-3 * nt)
    coords = storage.batch_coords(t, x, v, rules)
    second = coords["distribution_function"][1]
    assert second[0] == ("space" if rules["space"] == "all" else "fourier_mode")
    # a mismatched array is refused with the coordinate it misses
    sc["fields"]["e"] = sc["fields"]["e"][:, :-1]
    with pytest.raises(ValueError, match="space"):
        storage.check_batch(sc, x, v, rules)

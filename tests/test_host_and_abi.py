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


def test_struct_layout_matches_header(lib_path):
    from vlapy_gb300 import _lib
    src = "#include <stdio.h>\n#include \"vlagpu.h\"\nint main(){printf(\"%zu %zu %zu\", sizeof(vg_run_desc), sizeof(vg_history), sizeof(vg_pulse));}"
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
    assert [int(x) for x in out] == [ctypes.sizeof(_lib.VgRunDesc), ctypes.sizeof(_lib.VgHistory),
                                     ctypes.sizeof(_lib.VgPulse)]


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


def test_unknown_names_raise_not_implemented():
    from vlapy_gb300.core import collisions
    with pytest.raises(NotImplementedError):
        collisions.check_names({"type": "bgk", "solver": "batched_tridiagonal"})
    with pytest.raises(NotImplementedError):
        collisions.check_names({"type": "dg", "solver": "lu"})
    assert collisions.check_names({"type": "dg", "solver": "naive"}) == ("dg", "naive")


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
    np.testing.assert_allclose(p["w_epw"] + 1j * p["nu_ld"], vo.epw_root(0.3), rtol=1e-14)

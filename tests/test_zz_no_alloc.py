"""vg_field_solve_noalloc: the field solve for callers that cannot allocate
device memory (their memory belongs to another allocator, or they cannot
take the synchronisation of cudaMalloc/cudaFree).  It keeps its scratch in a
static device array; this checks it against the plan-based vg_field_solve,
called twice in a row through the C ABI.  Collected last on purpose."""

import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import vlapy_oracle as vo  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the FP64 parity tolerance of the other GPU tests


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import _lib
    return _lib.load()


def _case(nx, nv, seed):
    rng = np.random.default_rng(seed)
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / 0.3, nx)
    dv, v, kv = vo.velocity_axis(6.4, nv)
    f = vo.maxwellian(nx, nv, 6.4) * (1.0 + 1e-3 * np.cos(0.3 * x + rng.uniform(0, 6)))[:, None]
    drv = 1e-3 * np.sin(0.3 * x)
    return f, drv, (x, v, kx, kv, inv, dx, dv)


@pytest.mark.parametrize("nx,nv", [(32, 512), (96, 256), (8192, 16), (64, 16384), (5, 9)])
def test_noalloc_field_solve_matches_plan(lib, nx, nv):
    from vlapy_gb300._lib import check
    from vlapy_gb300.plan import Plan, ptr, stream_handle
    f, drv, (x, v, kx, kv, inv, dx, dv) = _case(nx, nv, nx + nv)
    plan = Plan(nx, nv, x, v, kx, kv, inv, dx, dv)
    ft = torch.as_tensor(f, device="cuda")
    dt_ = torch.as_tensor(drv, device="cuda")
    inv_t = torch.as_tensor(inv, device="cuda")
    for driver in (dt_, None):
        ref = torch.empty(nx, dtype=torch.float64, device="cuda")
        plan.field_solve(ft, driver, ref)
        for _ in range(2):  # two calls in a row share (and overwrite) the static scratch
            out = torch.full((nx,), float("nan"), dtype=torch.float64, device="cuda")
            check(lib.vg_field_solve_noalloc(ptr(ft), nx, nv, C.c_double(dv), ptr(inv_t), ptr(driver), ptr(out),
                                             stream_handle()), "field solve noalloc")
            torch.cuda.synchronize()
            a, b = out.cpu().numpy(), ref.cpu().numpy()
            assert np.linalg.norm(a - b) <= TOL * np.linalg.norm(b)


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    from vlapy_gb300._lib import VG_ERR_ARG
    from vlapy_gb300.plan import ptr, stream_handle
    f = torch.zeros((16384, 2), dtype=torch.float64, device="cuda")
    inv = torch.zeros(16384, dtype=torch.float64, device="cuda")
    e = torch.zeros(16384, dtype=torch.float64, device="cuda")
    st = lib.vg_field_solve_noalloc(ptr(f), 16384, 2, C.c_double(0.1), ptr(inv), None, ptr(e), stream_handle())
    assert st == VG_ERR_ARG
    assert b"nx <= 8192" in lib.vg_last_error()
    # one velocity point past the limit (the sizes are checked before any launch)
    f2 = torch.zeros((2, 16385), dtype=torch.float64, device="cuda")
    st = lib.vg_field_solve_noalloc(ptr(f2), 2, 16385, C.c_double(0.1), ptr(inv), None, ptr(e), stream_handle())
    assert st == VG_ERR_ARG
    assert b"nv <= 16384" in lib.vg_last_error() or b"nv=16385" in lib.vg_last_error()


def test_noalloc_on_a_second_stream(lib):
    """After the set-up call, a call on another stream (ordered after the
    first by the caller, as the shared scratch requires) gives the same field."""
    from vlapy_gb300._lib import check
    from vlapy_gb300.plan import Plan, ptr, stream_handle
    nx, nv = 64, 1024
    f, drv, (x, v, kx, kv, inv, dx, dv) = _case(nx, nv, 7)
    plan = Plan(nx, nv, x, v, kx, kv, inv, dx, dv)
    ft, dt_, inv_t = (torch.as_tensor(a, device="cuda") for a in (f, drv, inv))
    ref = torch.empty(nx, dtype=torch.float64, device="cuda")
    plan.field_solve(ft, dt_, ref)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    out = torch.full((nx,), float("nan"), dtype=torch.float64, device="cuda")
    with torch.cuda.stream(s):
        check(lib.vg_field_solve_noalloc(ptr(ft), nx, nv, C.c_double(dv), ptr(inv_t), ptr(dt_), ptr(out),
                                         stream_handle(s)), "field solve noalloc")
    torch.cuda.synchronize()
    a, b = out.cpu().numpy(), ref.cpu().numpy()
    assert np.linalg.norm(a - b) <= TOL * np.linalg.norm(b)


def test_noalloc_call_captured_in_a_graph(lib):
    """After the set-up call, a call copies nothing from host memory and only
    launches kernels on the caller's stream, so it can be recorded into a CUDA
    graph: two replays on new inputs give the plan-based field each time."""
    from vlapy_gb300._lib import check
    from vlapy_gb300.plan import Plan, ptr
    nx, nv = 64, 512
    f, drv, (x, v, kx, kv, inv, dx, dv) = _case(nx, nv, 11)
    plan = Plan(nx, nv, x, v, kx, kv, inv, dx, dv)
    ft, dt_, inv_t = (torch.as_tensor(a, device="cuda") for a in (f, drv, inv))
    out = torch.zeros(nx, dtype=torch.float64, device="cuda")
    check(lib.vg_field_solve_noalloc(ptr(ft), nx, nv, C.c_double(dv), ptr(inv_t), ptr(dt_), ptr(out),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream)), "set-up call")
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            st = lib.vg_field_solve_noalloc(ptr(ft), nx, nv, C.c_double(dv), ptr(inv_t), ptr(dt_), ptr(out),
                                            C.c_void_p(s.cuda_stream))
    assert st == 0, lib.vg_last_error()
    ref = torch.empty(nx, dtype=torch.float64, device="cuda")
    for seed in (12, 13):
        f2, drv2, _ = _case(nx, nv, seed)
        ft.copy_(torch.as_tensor(f2))
        dt_.copy_(torch.as_tensor(drv2))
        out.fill_(float("nan"))
        graph.replay()
        plan.field_solve(ft, dt_, ref)
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.linalg.norm(a - b) <= TOL * np.linalg.norm(b), seed

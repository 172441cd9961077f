"""Learned coarse-velocity corrector (vg_corr_*) against its CPU oracle.

Forward pass and gradients are compared with the torch float64 oracle in two
ways: with bfloat16 rounding emulated at the kernels' rounding points (tight
tolerance: only FP32-vs-FP64 accumulation differs) and as the plain float64
network under autograd (loose tolerance: the BF16 quantisation itself)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import corrector_oracle as co  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_loaded():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import _lib
    _lib.load()


def random_params(seed):
    from vlapy_gb300.corrector import init_params
    rng = np.random.default_rng(seed)
    p = init_params(seed)
    d = co.unpack(p)
    # a live last layer, so every gradient is non-zero
    d["W4"][:] = torch.as_tensor(rng.uniform(-0.1, 0.1, (1, co.HID, 5)))
    d["b4"][:] = 0.01
    return co.pack(d)


def random_rows(rows, seed, with_prev=False):
    rng = np.random.default_rng(seed)
    v = -6.4 + 0.1 * (np.arange(128) + 0.5)
    m = np.exp(-v ** 2 / 2)
    amp = 10.0 ** rng.uniform(-6, -2, (rows, 1))
    g = amp * m[None, :] * (np.cos(rng.uniform(1, 8, (rows, 1)) * v[None, :] + rng.uniform(0, 6, (rows, 1)))
                            + 0.3 * rng.standard_normal((rows, 128)))
    # a fixed linear correction: 0.02 x the discrete second difference along v
    gp = np.pad(g, ((0, 0), (1, 1)))
    corr = 0.02 * (gp[:, :-2] - 2 * g + gp[:, 2:])
    feat = co_nu_feature(10.0 ** rng.uniform(-5, -2, rows))
    out = (g.astype(np.float32), (g + corr).astype(np.float32), feat.astype(np.float32))
    if with_prev:
        prev = g + 0.05 * np.roll(g, 1, axis=1) + 1e-3 * amp * rng.standard_normal((rows, 128))
        out = out + (prev.astype(np.float32),)
    return out


def co_nu_feature(nu):
    from vlapy_gb300.corrector import nu_feature
    return nu_feature(nu)


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.parametrize("engine", ["tcgen05", "mma.sync"])
@pytest.mark.parametrize("rows,group,modes", [(1, 0, 0), (77, 0, 0), (1000, 0, 32), (960, 64, 32), (64, 64, 0),
                                              (90, 3, 64), (128, 64, 1)])
def test_forward_matches_oracle(rows, group, modes, engine):
    from vlapy_gb300.corrector import Corrector
    p = random_params(1)
    g, _, feat, prev = random_rows(rows, rows, with_prev=True)
    if rows == 77:
        prev = None  # the previous-state channel left empty
    tau = 0.05
    corr = Corrector(1024, params=p, tau=tau, protect_modes=modes)
    corr.set_engine(engine)
    gt, ft = torch.as_tensor(g, device="cuda"), torch.as_tensor(feat, device="cuda")
    pt = None if prev is None else torch.as_tensor(prev, device="cuda")
    out = corr.apply(gt, prev=pt, feat=ft, group_rows=group).cpu().numpy().astype(np.float64)
    ref_e = co.apply(p, g, feat, 6.4, tau, emulate=True, group_rows=group, protect_modes=modes, prev=prev)
    ref_x = co.apply(p, g, feat, 6.4, tau, emulate=False, group_rows=group, protect_modes=modes, prev=prev)
    # compare the corrections themselves (out - g), not the rows; the output
    # rows are FP32, so a correction near the rounding of g is resolved only
    # to ~1e-7 |g| (the 1e-6 floor below)
    gn = np.linalg.norm(g.astype(np.float64))
    assert np.linalg.norm((out - g) - (ref_e - g)) <= 2e-3 * np.linalg.norm(ref_e - g) + 1e-6 * gn
    assert np.linalg.norm((out - g) - (ref_x - g)) <= 0.1 * np.linalg.norm(ref_x - g) + 1e-6 * gn
    # the cap: no corrected row deviation is longer than the uncorrected one
    d = co.deviation(g, group).numpy().astype(np.float64)
    dn = d + (out - g)
    assert np.all(np.linalg.norm(dn, axis=1) <= np.linalg.norm(d, axis=1) * (1 + 1e-5) + 1e-30)
    # the protected modes of each row's deviation are untouched
    if modes:
        lo = np.fft.rfft(dn, axis=1)[:, :modes] - np.fft.rfft(d, axis=1)[:, :modes]
        scale_lo = np.abs(np.fft.rfft(d, axis=1)).max(axis=1, keepdims=True)
        assert np.all(np.abs(lo) <= 1e-5 * scale_lo)
    # in place: g_out aliasing g
    corr.apply(gt, prev=pt, feat=ft, out=gt, group_rows=group)
    np.testing.assert_array_equal(gt.cpu().numpy(), out.astype(np.float32))
    corr.check_status()


def test_engines_agree_on_many_rows():
    """The fused tcgen05 forward and the per-layer mma.sync kernels see the
    same BF16 operands; only FP32 accumulation order and rare BF16 rounding
    flips of the activations separate them."""
    from vlapy_gb300.corrector import Corrector
    p = random_params(5)
    rows = 64 * 300  # more rows than SMs: every persistent CTA loops
    g, _, feat, prev = random_rows(rows, 9, with_prev=True)
    gt, ft, pt = (torch.as_tensor(a, device="cuda") for a in (g, feat, prev))
    corr = Corrector(rows, params=p, tau=0.05)
    a = corr.apply(gt, prev=pt, feat=ft, group_rows=64)
    corr.set_engine("mma.sync")
    b = corr.apply(gt, prev=pt, feat=ft, group_rows=64)
    corr.check_status()
    da, db = (a - gt).double(), (b - gt).double()
    assert float(torch.linalg.norm(da - db) / torch.linalg.norm(db)) <= 1e-3


@pytest.mark.parametrize("engine", ["tcgen05", "mma.sync"])
@pytest.mark.parametrize("group,modes", [(0, 0), (60, 32), (60, 0)])
def test_gradients_match_oracle(group, modes, engine):
    """Loss and every parameter's gradient against the CPU oracle, for the
    training layers on either engine (tcgen05: forward, data-gradient and
    weight-gradient kernels per layer; mma.sync: the legacy kernels)."""
    from vlapy_gb300.corrector import Corrector
    p = random_params(2)
    rows = 300
    g, t, feat, prev = random_rows(rows, 3, with_prev=True)
    tau = 2e-3
    corr = Corrector(rows, params=p, tau=tau, protect_modes=modes)
    corr.set_engine(engine)
    gt, tt, ft, pt = (torch.as_tensor(a, device="cuda") for a in (g, t, feat, prev))
    loss, grad = corr.gradients(gt, tt, prev=pt, feat=ft, group_rows=group)
    loss_e, grad_e = co.loss_and_grads(p, g, feat, t, 6.4, tau, emulate=True, group_rows=group, protect_modes=modes,
                                       prev=prev)
    loss_x, grad_x = co.loss_and_grads(p, g, feat, t, 6.4, tau, emulate=False, group_rows=group,
                                       protect_modes=modes, prev=prev)
    assert abs(loss - loss_e) <= 1e-4 * loss_e
    assert abs(loss - loss_x) <= 1e-2 * loss_x
    o = 0
    for name, shape in co.SHAPES:
        n = int(np.prod(shape))
        a, e, x = grad[o:o + n], grad_e[o:o + n], grad_x[o:o + n]
        if name == "W1":  # input channels 4..15 carry zeros: their gradient is exactly zero
            a3 = a.reshape(shape)
            assert np.all(a3[:, 4:, :] == 0)
        if name == "b4" and modes:
            # the projected loss is blind to a constant output: the exact b4
            # gradient is zero, and what remains is the sum of the BF16
            # rounding errors of the loss gradient, noise of no fixed value
            assert abs(a[0]) <= 1e-2 * np.abs(grad_x).max()
            assert abs(e[0]) <= 1e-2 * np.abs(grad_x).max()
        else:
            # emulated rounding: only FP32 accumulation order and rare BF16
            # rounding flips differ; plain FP64: the BF16 quantisation itself
            assert rel(a, e) <= 5e-3, (name, rel(a, e))
            assert rel(a, x) <= 0.15, (name, rel(a, x))
        o += n


def test_training_engines_agree_on_many_rows():
    """The tcgen05 training layers against the mma.sync ones on more rows than
    the persistent CTAs' slots (every slot loops) and than the weight
    gradient's row chunks hold (every chunk accumulates many rows in TMEM).
    Both see the same BF16 operands, add K = 16 partial products into FP32
    in the same order and reduce the row chunks in the same order: the
    losses and gradients are bit for bit the same."""
    from vlapy_gb300.corrector import Corrector
    p = random_params(6)
    rows = 64 * 200
    g, t, feat, prev = random_rows(rows, 12, with_prev=True)
    gt, tt, ft, pt = (torch.as_tensor(a, device="cuda") for a in (g, t, feat, prev))
    corr = Corrector(rows, params=p, tau=2e-3, protect_modes=32)
    la, ga = corr.gradients(gt, tt, prev=pt, feat=ft, group_rows=64)
    corr.check_status()
    corr.set_engine("mma.sync")
    lb, gb = corr.gradients(gt, tt, prev=pt, feat=ft, group_rows=64)
    assert la == lb
    np.testing.assert_array_equal(ga, gb)


def test_training_fits_a_fixed_filter():
    """Adam on a synthetic target (a fixed smooth correction) drives the loss down."""
    from vlapy_gb300.corrector import Corrector
    rows = 4096
    g, t, feat = random_rows(rows, 11)
    gt, tt, ft = (torch.as_tensor(a, device="cuda") for a in (g, t, feat))
    s = np.sqrt(np.mean(g.astype(np.float64) ** 2, axis=1)) + 1e-30
    tau = float(np.sqrt(np.mean(((t - g) / s[:, None]) ** 2)))
    corr = Corrector(rows, tau=tau, protect_modes=0)
    first = corr.loss(gt, tt, feat=ft)
    assert abs(first - 1.0) < 0.05  # untrained: zero output, loss = mean(want^2) = 1
    for _ in range(300):
        corr.train_step(gt, tt, feat=ft, lr=2e-3)
    last = corr.loss(gt, tt, feat=ft)
    assert last < 0.05 * first, (first, last)


def test_set_params_roundtrip_and_errors():
    from vlapy_gb300.corrector import Corrector
    p = random_params(4)
    corr = Corrector(16, params=p)
    np.testing.assert_array_equal(corr.params, p)
    with pytest.raises(ValueError):
        corr.apply(torch.zeros((17, 128), device="cuda"))
    with pytest.raises(ValueError):
        corr.apply(torch.zeros((4, 64), device="cuda"))
    with pytest.raises(ValueError):
        Corrector(16, params=p[:-1])
    with pytest.raises(ValueError):
        corr.apply(torch.zeros((12, 128), device="cuda"), group_rows=5)

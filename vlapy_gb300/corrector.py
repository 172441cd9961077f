"""Learned coarse-velocity corrector for the batched sweep (no reference
counterpart).

A run on a coarse velocity grid (nv = 128 at the same vmax) is cheap but
under-resolves filamentation and the velocity-space diffusion of the
Fokker-Planck step.  After each coarse step a small 1-D conv net along v
(libvlagpu vg_corr_*: four conv1d layers, kernel 5, 64 channels, BF16 tensor
cores with FP32 accumulation) adds a correction to every x row:

    c = P(s * tau * net(d / s, v / vmax, nu_feature(nu), d_prev / s)),
    g <- m + (d - Pd) + (Pd + c) * min(1, |Pd| / |Pd + c|),

m the run's x-mean, d = g - m, d_prev the same before the coarse step
(the pair shows which way each filament moves in kv; the x-mean carries the coarse grid's slow
drift of the Maxwellian under the collision operator, which does not reach
the field), s the RMS of d and tau a global scale fixed from the training
data.  P removes the v-Fourier modes |m| < 56 of the row from the
correction: the one-step difference between the grids sits almost entirely
near the coarse Nyquist mode (filaments that the fine grid carries out of
the coarse band and that the coarse grid would alias back: its recurrence),
while the lower modes carry the density and hence the field, which the
coarse grid already gets right and which a network's small errors would
only disturb.  On held-out rollouts against fine FP64 runs the damping rate
gets monotonically better the more modes are protected (8 to 60 tried); 56
keeps the uncorrected grid's damping accuracy and most of the field-energy
gain.  The cap keeps the corrected high part of each row no
larger in L2 norm than the coarse step made it, so repeated corrections
cannot feed energy into a run.
The network is trained, with the library's own forward, backward and Adam
kernels, to map the coarse step of a restricted fine state onto the
restriction of the fine step.  Restriction is spectral truncation of the
fine v-spectrum to the coarse one at equal vmax, sampled at the coarse cell
centres (``restriction_matrix``).

Training data come from the method itself: a fine sweep (nv = 1024) of runs
drawn like the sweep workload, with snapshot pairs every ``every`` steps.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from ._lib import check
from .initializers import initialize_distribution
from .plan import ptr, require_cuda, stream_handle
from .sweep import Sweep, sweep_config

NV = 128
C_IN, HID = 16, 64
SHAPES = [("W1", (HID, C_IN, 5)), ("b1", (HID,)), ("W2", (HID, HID, 5)), ("b2", (HID,)),
          ("W3", (HID, HID, 5)), ("b3", (HID,)), ("W4", (1, HID, 5)), ("b4", (1,))]
N_INPUTS = 4  # d / s, v / vmax, collision-rate feature, d_prev / s
PROTECT_MODES = 56  # v-Fourier modes |m| < 56 of the 128-point row are never corrected


def nu_feature(nu):
    """Collision-rate input channel: 0 for collisionless runs, about 1 at nu = 1e-2."""
    return np.log10(1.0 + np.asarray(nu, dtype=np.float64) / 1e-5) / 3.0


def init_params(seed=0):
    """PyTorch-style uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights over the
    used input channels; the last layer starts at zero, so the untrained
    network leaves the coarse step unchanged."""
    rng = np.random.default_rng(seed)
    out = []
    for name, shape in SHAPES:
        if name == "W1":
            w = np.zeros(shape)
            bound = 1.0 / math.sqrt(N_INPUTS * 5)
            w[:, :N_INPUTS, :] = rng.uniform(-bound, bound, (shape[0], N_INPUTS, 5))
        elif name in ("W4", "b4"):
            w = np.zeros(shape)
        elif name.startswith("W"):
            bound = 1.0 / math.sqrt(shape[1] * 5)
            w = rng.uniform(-bound, bound, shape)
        else:
            fan_in = (N_INPUTS if name == "b1" else HID) * 5
            bound = 1.0 / math.sqrt(fan_in)
            w = rng.uniform(-bound, bound, shape)
        out.append(w.reshape(-1))
    return np.concatenate(out).astype(np.float32)


def restriction_matrix(nv_fine, nv_coarse=NV):
    """[nv_coarse][nv_fine] float64: keep the v-Fourier modes |m| < nv_coarse/2
    of a fine row (the coarse Nyquist mode is dropped) and evaluate the
    truncated series at the coarse cell centres of the same [-vmax, vmax)."""
    r = nv_fine // nv_coarse
    if r * nv_coarse != nv_fine or r < 1:
        raise ValueError("nv_fine must be a multiple of nv_coarse")
    m = np.fft.fftfreq(nv_fine, 1.0 / nv_fine)
    keep = np.abs(m) < nv_coarse // 2
    # fine sample i sits at u = dv_f (i + 1/2); coarse sample j at dv_f (r j + r/2)
    i = np.arange(nv_fine)
    j = np.arange(nv_coarse)
    mk = m[keep]
    phase_f = np.exp(-2j * np.pi * np.outer(mk, i) / nv_fine)                      # forward DFT rows
    phase_c = np.exp(2j * np.pi * np.outer(r * j + (r - 1) / 2.0, mk) / nv_fine)   # evaluate at coarse centres
    return np.real(phase_c @ phase_f) / nv_fine


class Corrector:
    """Owns a vg_corrector (parameters, Adam state and activation buffers for
    up to max_rows rows).  Every call takes a batch of rows: ``g`` the state
    after the coarse step, ``prev`` the state before it, ``feat`` the
    collision-rate feature per row, ``target`` the training target, all
    contiguous CUDA float32; with ``group_rows`` > 0 the x-mean of each
    group of that many rows (one run) is taken out first."""

    def __init__(self, max_rows, params=None, seed=0, vmax=6.4, tau=1.0, protect_modes=PROTECT_MODES):
        require_cuda()
        self._lib = _lib.load()
        n = self._lib.vg_corr_num_params()
        p = init_params(seed) if params is None else np.ascontiguousarray(params, dtype=np.float32)
        if p.size != n:
            raise ValueError(f"expected {n} parameters, got {p.size}")
        h = C.c_void_p()
        check(self._lib.vg_corr_create(int(max_rows), int(protect_modes), float(vmax), float(tau), p.ctypes.data,
                                       C.byref(h)), "corrector create")
        self._h = h
        self.max_rows = int(max_rows)
        self.n_params = n
        self.vmax = float(vmax)
        self._tau = float(tau)
        self.protect_modes = int(protect_modes)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.vg_corr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def tau(self):
        return self._tau

    @tau.setter
    def tau(self, value):
        check(self._lib.vg_corr_set_tau(self._h, float(value)), "corrector tau")
        self._tau = float(value)

    def set_engine(self, engine):
        """"tcgen05" (default): the 5th-generation tensor cores, the fused
        forward for apply and one kernel per layer (forward, data gradient,
        weight gradient) for training; "mma.sync": the same layers on the
        legacy warp-level MMA."""
        code = {"tcgen05": 0, "mma.sync": 1}[engine]
        check(self._lib.vg_corr_set_engine(self._h, code), "corrector engine")

    def check_status(self):
        """Raise if a bounded wait of a tcgen05 kernel ran out (synchronises)."""
        flags = C.c_int32()
        check(self._lib.vg_corr_status(self._h, C.byref(flags)), "corrector status")

    @property
    def params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        check(self._lib.vg_corr_get_params(self._h, out.ctypes.data), "corrector params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        check(self._lib.vg_corr_set_params(self._h, p.ctypes.data), "corrector params")

    def _batch(self, g, prev=None, feat=None, target=None, group_rows=0, out=None):
        if not (isinstance(g, torch.Tensor) and g.is_cuda and g.dtype == torch.float32 and g.is_contiguous()
                and g.dim() == 2 and g.shape[1] == NV):
            raise ValueError("rows must be a contiguous CUDA float32 tensor [rows][128]")
        rows = g.shape[0]
        if rows > self.max_rows:
            raise ValueError(f"{rows} rows > max_rows {self.max_rows}")
        for t, shape in ((prev, (rows, NV)), (target, (rows, NV)), (out, (rows, NV)), (feat, (rows,))):
            if t is not None and not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32
                                      and t.is_contiguous() and tuple(t.shape) == shape):
                raise ValueError(f"expected a contiguous CUDA float32 tensor of shape {shape}")
        if group_rows < 0 or (group_rows and rows % group_rows):
            raise ValueError("group_rows must be 0 or divide the number of rows")
        return _lib.VgCorrBatch(ptr(g), ptr(prev), ptr(feat), ptr(target), rows, int(group_rows))

    def apply(self, g, prev=None, feat=None, out=None, group_rows=0, stream=None):
        """Corrected rows (out may be g itself)."""
        b = self._batch(g, prev, feat, None, group_rows, out)
        if out is None:
            out = torch.empty_like(g)
        check(self._lib.vg_corr_apply(self._h, C.byref(b), ptr(out), stream_handle(stream)), "corrector apply")
        return out

    def loss(self, g, target, prev=None, feat=None, group_rows=0, stream=None):
        b = self._batch(g, prev, feat, target, group_rows)
        out = C.c_double()
        check(self._lib.vg_corr_loss(self._h, C.byref(b), C.byref(out), stream_handle(stream)), "corrector loss")
        return out.value

    def gradients(self, g, target, prev=None, feat=None, group_rows=0, stream=None):
        """(loss, gradient float32 [n_params]) of one batch."""
        b = self._batch(g, prev, feat, target, group_rows)
        grad = np.empty(self.n_params, dtype=np.float32)
        out = C.c_double()
        check(self._lib.vg_corr_gradients(self._h, C.byref(b), grad.ctypes.data, C.byref(out),
                                          stream_handle(stream)), "corrector gradients")
        return out.value, grad

    def train_step(self, g, target, prev=None, feat=None, lr=1e-3, group_rows=0, want_loss=False, stream=None):
        b = self._batch(g, prev, feat, target, group_rows)
        out = C.c_double()
        check(self._lib.vg_corr_train_step(self._h, C.byref(b), float(lr), C.byref(out) if want_loss else None,
                                           stream_handle(stream)), "corrector train")
        return out.value if want_loss else None


def corrector_runs(n_runs, seed, nx=64):
    """Runs of the sweep distribution (k, amplitude, nu) at one nx; nv is set
    by the caller (fine or coarse)."""
    return [dict(r, nx=nx) for r in sweep_config(n_runs, seed=seed, nx_choices=(nx,), nv_choices=(1024,))]


class Pairing:
    """A fine sweep and its coarse twin (same runs, nv = 128) with the
    restriction between their packed states."""

    def __init__(self, runs, nv_fine=1024, vmax=6.4, dt=0.1):
        nx = {r["nx"] for r in runs}
        if len(nx) != 1:
            raise ValueError("all runs of a pairing share nx")
        self.nx = nx.pop()
        self.nv_fine = nv_fine
        self.fine = Sweep([dict(r, nv=nv_fine) for r in runs], vmax=vmax, dt=dt)
        self.coarse = Sweep([dict(r, nv=NV) for r in runs], vmax=vmax, dt=dt)
        self.rows = len(runs) * self.nx
        R = restriction_matrix(nv_fine, NV)
        self.Rt = torch.as_tensor(R.T.copy(), device="cuda")  # float64 [nf][nc]
        f0f = initialize_distribution(1, nv_fine, vmax)[0]
        f0c = initialize_distribution(1, NV, vmax)[0]
        # restricted background minus the coarse background: added to every row
        self.bg = torch.as_tensor(R @ f0f - f0c, device="cuda")
        nu = np.repeat([r["nu"] for r in runs], self.nx)
        self.row_feat = torch.as_tensor(nu_feature(nu), dtype=torch.float32, device="cuda")

    def restrict(self, g_fine):
        """Coarse deviations [rows][128] float32 of a packed fine state."""
        gf = g_fine.view(self.rows, self.nv_fine).to(torch.float64)
        return (gf @ self.Rt + self.bg[None, :]).to(torch.float32)


class PairData:
    """Training or evaluation rows of the corrector, all float32 CUDA
    [snapshots * runs * nx][128] (feat: one value per row): ``x`` the coarse
    step of the restricted fine state, ``prev`` that restricted state (the
    coarse step's input), ``target`` the restricted fine step."""

    def __init__(self, x, prev, target, feat, nx):
        self.x, self.prev, self.target, self.feat, self.nx = x, prev, target, feat, int(nx)

    @property
    def rows(self):
        return self.x.shape[0]

    def take(self, idx):
        return (self.x[idx].contiguous(), self.prev[idx].contiguous(), self.target[idx].contiguous(),
                self.feat[idx].contiguous())


def generate_pairs(runs, n_steps=2000, every=50, first=50, dt=0.1, vmax=6.4, stride=1):
    """Training pairs from fine runs: at steps first, first+every, ... the fine
    state is restricted and advanced `stride` coarse steps while the fine run
    advances `stride` fine steps and is restricted (the target); a network
    trained on them corrects every `stride` steps (run_corrected)."""
    pr = Pairing(runs, vmax=vmax, dt=dt)
    pr.fine.reset()
    xs, ps, ts = [], [], []
    n = 0
    ef = torch.empty(pr.fine.x_points, dtype=torch.float64, device="cuda")
    while True:
        nxt = first if n == 0 else n + every
        if nxt >= n_steps:
            break
        pr.fine.run_steps(nxt - n)
        n = nxt
        g, _ = pr.fine.get_state(e_out=ef)
        gc = pr.restrict(g)
        pr.coarse.set_state(gc.view(-1), ef)
        pr.coarse.run_steps(stride)
        x, _ = pr.coarse.get_state()
        pr.fine.run_steps(stride)
        n += stride
        g1, _ = pr.fine.get_state()
        xs.append(x.view(pr.rows, NV).clone())
        ps.append(gc)
        ts.append(pr.restrict(g1))
    feat = pr.row_feat.repeat(len(xs))
    return PairData(torch.cat(xs), torch.cat(ps), torch.cat(ts), feat, pr.nx)


def _batches(data, batch_runs, order=None):
    n_groups = data.rows // data.nx
    order = torch.arange(n_groups, device=data.x.device) if order is None else order
    for b in range(0, n_groups, batch_runs):
        grp = order[b:b + batch_runs]
        idx = (grp[:, None] * data.nx + torch.arange(data.nx, device=grp.device)[None, :]).reshape(-1)
        yield data.take(idx)


def evaluate(corr, data, batch_runs=128):
    """Mean loss over a data set (with zero network output it is the mean
    squared corrected part of the correction over tau^2)."""
    tot, cells = 0.0, 0
    for x, p, t, f in _batches(data, batch_runs):
        tot += corr.loss(x, t, p, f, group_rows=data.nx) * x.shape[0]
        cells += x.shape[0]
    return tot / cells


def output_scale(data, protect_modes=PROTECT_MODES, batch_runs=128):
    """tau: RMS over all rows of the corrected part (modes |m| >= M) of the
    correction in units of the row RMS, on the x-varying parts.  Measured
    with the loss kernel of an untrained network (zero output) at tau = 1."""
    probe = Corrector(batch_runs * data.nx, tau=1.0, protect_modes=protect_modes)
    try:
        return math.sqrt(evaluate(probe, data, batch_runs))
    finally:
        probe.close()


def train(corr, data, epochs=4, batch_runs=128, lr=1e-3, seed=0, log=None):
    """Adam over mini-batches of whole runs (batch_runs x nx rows, so that the
    x-means are taken inside the kernels), shuffled each epoch, learning rate
    halved per epoch.  Returns the mean sampled loss of each epoch."""
    gen = torch.Generator(device="cpu").manual_seed(seed)
    n_groups = data.rows // data.nx
    history = []
    for ep in range(epochs):
        perm = torch.randperm(n_groups, generator=gen).to(data.x.device)
        total, sampled = 0.0, 0
        for count, (x, p, t, f) in enumerate(_batches(data, batch_runs, perm)):
            if x.shape[0] < batch_runs * data.nx:
                continue
            want = (count % 50 == 0)
            l = corr.train_step(x, t, p, f, lr=lr * (0.5 ** ep), group_rows=data.nx, want_loss=want)
            if want:
                total += l
                sampled += 1
        history.append(total / max(1, sampled))
        if log:
            log(f"epoch {ep}: loss {history[-1]:.4e}")
    return history


def run_corrected(sweep, corr, nsteps, e_hist=None, series_hist=None, row0=0, stream=None, stride=1):
    """Advance a coarse sweep (all runs nv = 128, one nx) by nsteps steps,
    correcting every run in place after every `stride` steps (the stride of
    the network's training pairs); histories as Sweep.run_steps."""
    nx = {r["nx"] for r in sweep.runs}
    if len(nx) != 1 or any(r["nv"] != NV for r in sweep.runs):
        raise ValueError("the corrected path needs runs of one nx and nv = 128")
    nx = nx.pop()
    rows = sweep.cells // NV
    if rows > corr.max_rows:
        raise ValueError(f"{rows} rows > the corrector's max_rows {corr.max_rows}")
    g = sweep.state_view().view(rows, NV)
    prev = torch.empty_like(g)
    feat = getattr(sweep, "_corr_feat", None)
    if feat is None:
        feat = torch.as_tensor(np.repeat(nu_feature([r["nu"] for r in sweep.runs]), nx), dtype=torch.float32,
                               device="cuda")
        sweep._corr_feat = feat
    if stride < 1:
        raise ValueError("stride must be at least 1")
    for i in range(0, nsteps, stride):
        n = min(stride, nsteps - i)
        prev.copy_(g)
        sweep.run_steps(n, e_hist, series_hist, row0=row0 + i, stream=stream)
        corr.apply(g, prev, feat, out=g, group_rows=nx, stream=stream)
    corr.check_status()
    return sweep


def fine_reference(runs, nsteps=2000, vmax=6.4, dt=0.1):
    """Field-energy history [nsteps][runs] of the fine (nv = 1024) runs."""
    fine = Sweep([dict(r, nv=1024) for r in runs], vmax=vmax, dt=dt)
    fine.reset()
    eh, sh = fine.history(nsteps)
    fine.run_steps(nsteps, eh, sh)
    e2 = sh[:, :, 3].clone()
    fine.close()
    return e2


def rollout_error(corr, runs, e2_fine, vmax=6.4, dt=0.1, stride=1):
    """Per-run relative L2 error of the corrected coarse runs' field-energy
    history against the fine runs' (float64 CPU tensor [runs])."""
    nsteps = e2_fine.shape[0]
    sw = Sweep([dict(r, nv=NV) for r in runs], vmax=vmax, dt=dt)
    sw.reset()
    eh, sh = sw.history(nsteps)
    run_corrected(sw, corr, nsteps, eh, sh, stride=stride)
    e2 = sh[:, :, 3]
    err = torch.linalg.norm(e2 - e2_fine, dim=0) / torch.linalg.norm(e2_fine, dim=0)
    sw.close()
    return err.cpu()


def train_selected(data, val_runs, seeds=(0, 1, 2), epochs=4, batch_runs=128, lr=1e-3, max_rows=None,
                   protect_modes=PROTECT_MODES, log=None, stride=1):
    """Train one network per seed (initialisation and shuffling) and keep the
    one whose corrected coarse runs follow the fine runs best on validation
    runs (the mean field-energy-history error over 2000 steps).  Training one
    step at a time leaves the rollout quality of a network to chance; the
    validation runs are drawn apart from both the training and any held-out
    runs.  Returns (corrector, report)."""
    tau = output_scale(data, protect_modes=protect_modes)
    e2_fine = fine_reference(val_runs)
    rows = max(batch_runs * data.nx, len(val_runs) * data.nx, max_rows or 0)
    best, report = None, []
    for seed in seeds:
        corr = Corrector(rows, tau=tau, seed=seed, protect_modes=protect_modes)
        hist = train(corr, data, epochs=epochs, batch_runs=batch_runs, lr=lr, seed=seed)
        err = rollout_error(corr, val_runs, e2_fine, stride=stride)
        score = float(err.mean())
        report.append({"seed": seed, "train_loss": hist[-1], "val_field_energy_err_mean": score,
                       "val_within_1pct": float((err <= 0.01).double().mean())})
        if log:
            log(f"seed {seed}: validation field-energy error {score:.3e}")
        if best is None or score < best[0]:
            if best is not None:
                best[1].close()
            best = (score, corr)
        else:
            corr.close()
    return best[1], report

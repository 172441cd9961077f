"""What the trained corrector gains over the uncorrected coarse-velocity step.

Trains the network with the library's own kernels on pairs from 256 fine
runs (nv = 1024, seed 5) of the sweep distribution at nx = 64, then judges it
on 64 held-out runs (seed 6) against the fine runs:
- the one-step error on held-out pairs drops well below the uncorrected one;
- the field-energy history of corrected coarse runs is closer to the fine
  runs than that of uncorrected coarse runs, on average over the runs;
- the damping rate stays within 1% of the fine runs for the median run.
The fine runs are the FP32 batched sweep, which the sweep tests hold to the
FP64 oracle."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

NSTEPS = 2000


@pytest.fixture(scope="module")
def trained():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vlapy_gb300 import corrector as cm
    data = cm.generate_pairs(cm.corrector_runs(256, seed=5), n_steps=NSTEPS)
    tau = cm.output_scale(data)
    corr = cm.Corrector(64 * 64, tau=tau, seed=0)
    hist = cm.train(corr, data, epochs=4, batch_runs=64)
    return corr, hist


def test_one_step_error_drops_on_held_out_pairs(trained):
    from vlapy_gb300 import corrector as cm
    corr, hist = trained
    held = cm.generate_pairs(cm.corrector_runs(64, seed=6), n_steps=NSTEPS)
    zero = cm.Corrector(64 * 64, params=np.zeros(corr.n_params, np.float32), tau=corr.tau)
    base = cm.evaluate(zero, held, batch_runs=64)
    loss = cm.evaluate(corr, held, batch_runs=64)
    assert 0.5 < base < 2.0  # tau was set from the training pairs
    assert loss < 0.75 * base, (loss, base, hist)


def test_rollouts_against_fine_runs(trained):
    from vlapy_gb300 import corrector as cm
    from vlapy_gb300.diagnostics import damping_fit, mode_amplitude
    from vlapy_gb300.sweep import Sweep
    corr, _ = trained
    ev = cm.corrector_runs(64, seed=6)
    fine = Sweep([dict(r, nv=1024) for r in ev])
    coarse = Sweep([dict(r, nv=128) for r in ev])
    corrected = Sweep([dict(r, nv=128) for r in ev])
    out = []
    for sw in (fine, coarse):
        sw.reset()
        eh, sh = sw.history(NSTEPS)
        sw.run_steps(NSTEPS, eh, sh)
        out.append((eh, sh))
    corrected.reset()
    ek, sk = corrected.history(NSTEPS)
    cm.run_corrected(corrected, corr, NSTEPS, ek, sk)
    torch.cuda.synchronize()
    e2f, e2c, e2k = (s[:, :, 3].cpu().numpy() for s in (out[0][1], out[1][1], sk))
    assert np.isfinite(e2k).all()
    err_c = np.linalg.norm(e2c - e2f, axis=0) / np.linalg.norm(e2f, axis=0)
    err_k = np.linalg.norm(e2k - e2f, axis=0) / np.linalg.norm(e2f, axis=0)
    assert err_k.mean() < 0.5 * err_c.mean(), (err_k.mean(), err_c.mean())
    t = 0.1 * np.arange(1, NSTEPS + 1)
    rel = []
    for i in range(len(ev)):
        rf, _ = damping_fit(t, mode_amplitude(fine.e_of(out[0][0], i).cpu().numpy()), t_min=5.0, t_max=60.0)
        rk, _ = damping_fit(t, mode_amplitude(corrected.e_of(ek, i).cpu().numpy()), t_min=5.0, t_max=60.0)
        if np.isfinite(rf) and np.isfinite(rk):
            rel.append(abs(rk - rf) / abs(rf))
    assert len(rel) > 48
    assert np.median(rel) <= 0.01, np.median(rel)

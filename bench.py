"""Benchmark of the VlaPy time step on GB300 (one JSON line on rank 0).

A "step" is one full time step (VP step, Fokker-Planck step, storage step) of
the named workload.  ``value`` is phase-space cell-updates per second timed on
the device with CUDA events around a CUDA graph of K steps (inputs resident in
HBM); ``e2e`` is the same metric through the C-ABI entry point with the
step's inputs copied from pinned host memory and its stored fields/series
read back every step.  ``roofline`` is the dominant kernel's algorithmic
bytes per launch over its CUDA-event launch time in a profiled pass.
``--impl reference`` times the CPU oracle (a NumPy restatement of the
reference path) on the host cores instead.

Workloads (synthetic inputs of the reference's shapes; no datasets involved):
  sweep   4096 independent runs (seeded: nx in {32,64,128}, nv in {256,512,1024},
          k ~ U[0.25,0.45], amplitude 10^U[-6,-2], nu 10^U[-5,-2] with 25% zero,
          DG collisions, vmax=6.4, dt=0.1), all advanced by every launch
  large   nx=4096, nv=8192, xmax=2pi/0.3, vmax=8, two-stream f, nu=1e-4 DG, dt=0.05
  driven  nx=64, nv=1024, k=0.3, vmax=6.4, sin^2-enveloped driver, nu=1e-3 DG, dt=0.1
  landau  nx=32, nv=512, k=0.3, vmax=6.4, A=1e-4, nu=0, dt=0.1
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SWEEP_STEPS = 2000  # steps of one sweep run (the workload's run length)

WORKLOADS = {
    "sweep": dict(kind="sweep", n_runs=4096, seed=20261203, vmax=6.4, dt=0.1),
    "large": dict(nx=4096, nv=8192, k=0.3, vmax=8.0, dt=0.05, nu=1e-4, op="dg", kind="two-stream"),
    "driven": dict(nx=64, nv=1024, k=0.3, vmax=6.4, dt=0.1, nu=1e-3, op="dg", kind="driven"),
    "landau": dict(nx=32, nv=512, k=0.3, vmax=6.4, dt=0.1, nu=0.0, op="dg", kind="landau"),
    # the learned path's network alone: one correction of 2048 coarse runs x 64 x rows
    "corrector": dict(kind="corrector", n_runs=2048, nx=64, vmax=6.4),
    # the plain FP64 GPU method on the sweep's runs: the batched FP64 step alone
    "fp64sweep": dict(kind="fp64sweep", n_runs=4096, seed=20261203, vmax=6.4, dt=0.1),
    # one Adam step of the corrector on a training batch of 128 runs x 64 rows
    "corrector-train": dict(kind="corrector-train", n_runs=128, nx=64, vmax=6.4),
}



def corrector_issued_flops(rows, nv):
    """FLOPs the tensor cores execute for one corrector apply: per row of nv
    positions, layer 1 (its 5 taps x 4 channels folded into K = 32, N = 64),
    layers 2 and 3 (5 taps, K = N = 64) and layer 4 (its 5 taps as N = 16,
    K = 64)."""
    return 2.0 * rows * nv * (32 * 64 + 5 * 64 * 64 + 5 * 64 * 64 + 64 * 16)

def initial_state(w, seed=4):
    """Initial f of a workload (host, float64)."""
    from vlapy_gb300 import initializers as I
    nx, nv, k, vmax = w["nx"], w["nv"], w["k"], w["vmax"]
    dx, x, kx, inv = I.initialize_spatial_quantities(0.0, 2 * np.pi / k, nx)
    dv, v, kv = I.initialize_velocity_quantities(vmax, nv)
    if w["kind"] == "two-stream":
        rng = np.random.default_rng(seed)
        ph = rng.uniform(0, 2 * np.pi, 16)
        m = np.arange(1, 17)
        pert = 1e-3 * np.cos(m[None, :] * k * x[:, None] + ph[None, :]).sum(axis=1)
        fv = 0.5 * (np.exp(-((v - 3.0) ** 2) / 2.0) + np.exp(-((v + 3.0) ** 2) / 2.0))
        fv = fv / np.trapezoid(fv, dx=dv)
        f = fv[None, :] * (1.0 + pert)[:, None]
    elif w["kind"] == "driven":
        f = I.initialize_distribution(nx, nv, vmax)
    else:
        f = I.initialize_distribution(nx, nv, vmax) * (1.0 + 1e-4 * np.cos(k * x))[:, None]
    return dict(x=x, v=v, kx=kx, kv=kv, inv=inv, dx=dx, dv=dv, f=f)


def pulses_of(w):
    if w["kind"] != "driven":
        return []
    from vlapy_gb300 import dispersion
    wr = float(np.real(dispersion.get_roots_to_electrostatic_dispersion(1.0, 1.0, w["k"])))
    return [{"k0": w["k"], "w0": wr, "a0": 1e-2, "t_L": 0.0, "t_R": 100.0, "envelope": 1}]


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", "vg_clocks_%d_%d.csv" % (os.getpid(), index))

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, flag in enumerate(r[2]) if flag.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# DRAM bytes of the sweep row pass per cell (dram__bytes_read.sum +
# dram__bytes_write.sum), measured by ncu on the three full row-pass launches
# of the 4096-run sweep (one per nv class; 179,806,208 cells in all):
# 256: 106.42 + 53.45 MB, 512: 210.23 + 159.97 MB, 1024: 405.17 + 348.15 MB.
ROW_PASS_DRAM_BYTES_PER_CELL = (106419968 + 53376768 + 210321664 + 154533632 + 404892416 + 364435712) / 179806208


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_gpu(args, w, rank, world):
    import torch
    from vlapy_gb300 import _lib
    from vlapy_gb300.plan import Plan, history_struct

    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    _lib.load()
    st = initial_state(w)
    nx, nv = w["nx"], w["nv"]
    fp32 = args.precision == "fp32-deltaf"
    f_bg = st["f"].mean(axis=0)
    plan = Plan(nx, nv, st["x"], st["v"], st["kx"], st["kv"], st["inv"], st["dx"], st["dv"], dt=w["dt"],
                nu=w["nu"], collision=w["op"] if w["nu"] > 0 else "none", pulses=pulses_of(w),
                precision=args.precision, f_background=f_bg if fp32 else None)

    def initial():
        if fp32:
            return torch.as_tensor((st["f"] - f_bg[None, :]).astype(np.float32), device=dev).contiguous()
        return torch.as_tensor(st["f"], dtype=torch.float64, device=dev).contiguous()
    dev = torch.device("cuda")
    K, W = args.steps, args.warmup
    nt = W + K + args.prof_steps
    dt = w["dt"]
    tb_host = dt * np.arange(nt)
    drv_host = np.zeros((nt, nx))
    if pulses_of(w):
        from vlapy_gb300 import field_driver
        pd = field_driver.PulseDriver(st["x"], {"p": dict(pulses_of(w)[0], envelope="sin2")})
        drv_host = field_driver.make_driver_array(pd, st["x"], tb_host)
    f = initial()
    e = torch.zeros(nx, dtype=torch.float64, device=dev)
    tb = torch.as_tensor(tb_host, device=dev)
    db = torch.as_tensor(drv_host, device=dev)
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device=dev)  # noqa: E731
    storage = {"stored_f": torch.zeros((nt, 2, nv), dtype=torch.complex64, device=dev),
               "fields": {k: z(nt, nx) for k in ("e", "driver", "n", "j", "T", "q", "fv4", "vN")},
               "series": {k: z(nt) for k in ("mean_n", "mean_j", "mean_T", "mean_e2", "mean_de2",
                                             "mean_f2", "mean_flogf")}}
    hist = history_struct(storage, nx, 2)
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        plan.run_steps(f, e, hist, tb, db, 0, W, use_graph=False, stream=stream)
        # capture the K timed steps once, then replay it (a second capture
        # key would be a second graph; reuse the warm one for the timing)
        plan.run_steps(f, e, hist, tb, db, W, K, use_graph=True, stream=stream)
    torch.cuda.synchronize()
    f.copy_(initial())
    e.zero_()
    with torch.cuda.stream(stream):
        plan.run_steps(f, e, hist, tb, db, 0, W, use_graph=False, stream=stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    with torch.cuda.stream(stream):
        plan.run_steps(f, e, hist, tb, db, W, K, use_graph=True, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if not torch.isfinite(e).all():
        raise RuntimeError("non-finite field after the timed steps")
    # profiled pass: per-kernel launch times (graph bypassed)
    plan.profile(True)
    with torch.cuda.stream(stream):
        plan.run_steps(f, e, hist, tb, db, W + K, args.prof_steps, use_graph=False, stream=stream)
    prof = plan.profile_read()
    plan.profile(False)
    # e2e: per step, pinned host time/driver in, stored fields + series out
    e2e = run_e2e(plan, f, e, storage, hist, tb_host, drv_host, W, K, stream, torch)
    return ms, prof, clk, e2e, plan


def run_e2e(plan, f, e, storage, hist, tb_host, drv_host, W, K, stream, torch):
    nx = plan.nx
    dev = torch.device("cuda")
    pin_t = torch.as_tensor(tb_host).pin_memory()
    pin_d = torch.as_tensor(drv_host).pin_memory()
    tb = torch.empty_like(pin_t, device=dev)
    db = torch.empty_like(pin_d, device=dev)
    out_fields = torch.empty((8, nx), dtype=torch.float64).pin_memory()
    out_series = torch.empty(7, dtype=torch.float64).pin_memory()
    fk = ("e", "driver", "n", "j", "T", "q", "fv4", "vN")
    sk = ("mean_n", "mean_j", "mean_T", "mean_e2", "mean_de2", "mean_f2", "mean_flogf")
    h2d = pin_t[0].numel() * 8 + pin_d[0].numel() * 8
    d2h = out_fields.numel() * 8 + out_series.numel() * 8
    # the step's inputs go in on the compute stream; its stored fields and
    # series come out on a copy stream while the next step runs, into one of
    # two pinned buffers, and the host waits for every step's result one step
    # later (the last one before the clock stops)
    out_f = [out_fields, torch.empty_like(out_fields).pin_memory()]
    out_s = [out_series, torch.empty_like(out_series).pin_memory()]
    copy_stream = torch.cuda.Stream()
    ev_step = [torch.cuda.Event() for _ in range(2)]
    ev_copy = [torch.cuda.Event() for _ in range(2)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for n, i in enumerate(range(W, W + K)):
        b = n % 2
        with torch.cuda.stream(stream):
            tb[i].copy_(pin_t[i], non_blocking=True)
            db[i].copy_(pin_d[i], non_blocking=True)
            plan.run_steps(f, e, hist, tb, db, i, 1, use_graph=False, stream=stream)
        ev_step[b].record(stream)
        copy_stream.wait_event(ev_step[b])
        if n >= 2:
            ev_copy[b].synchronize()  # the host buffer b is free again
        with torch.cuda.stream(copy_stream):
            for q, k in enumerate(fk):
                out_f[b][q].copy_(storage["fields"][k][i], non_blocking=True)
            for q, k in enumerate(sk):
                out_s[b][q:q + 1].copy_(storage["series"][k][i:i + 1], non_blocking=True)
        ev_copy[b].record(copy_stream)
        if n > 0:
            ev_copy[1 - b].synchronize()
    ev_copy[(K - 1) % 2].synchronize()
    t1 = time.perf_counter()
    return (t1 - t0), h2d, d2h


def run_sweep_gpu(args, w, rank, world, global_rank=0):
    import torch
    from vlapy_gb300 import _lib
    from vlapy_gb300.replicas import shard_seed
    from vlapy_gb300.sweep import Sweep, sweep_config

    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    _lib.load()
    # each rank advances its own shard of the sweep (weak scaling)
    runs = sweep_config(w["n_runs"], shard_seed(w["seed"], global_rank))
    sw = Sweep(runs, vmax=w["vmax"], dt=w["dt"])
    K, W = args.steps, args.warmup
    eh, sh = sw.history(K)
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        sw.reset(stream)
        sw.run_steps(W, use_graph=False, stream=stream)
        sw.run_steps(K, eh, sh, use_graph=True, stream=stream)  # capture
        sw.reset(stream)
        sw.run_steps(W, use_graph=False, stream=stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    with torch.cuda.stream(stream):
        sw.run_steps(K, eh, sh, use_graph=True, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if not torch.isfinite(eh).all():
        raise RuntimeError("non-finite field in the sweep history")
    sw.profile(True)
    with torch.cuda.stream(stream):
        sw.run_steps(args.prof_steps, eh, sh, use_graph=False, stream=stream)
    prof = sw.profile_read()
    sw.profile(False)
    # e2e: the K steps in one run_steps call through the C ABI (one replay of
    # the graph that an untimed call with the same arguments captured), every
    # step's e row and series taken to pinned host memory by a copy stream as
    # soon as the step has stored them (the graph records a CUDA event after
    # each step), and the host waiting for each step's result in turn while
    # the later steps run
    events = [torch.cuda.Event() for _ in range(K)]
    sw.set_step_events(events)
    out_e = [torch.empty(sw.x_points, dtype=torch.float64).pin_memory()]
    out_s = [torch.empty((sw.n_runs, 7), dtype=torch.float64).pin_memory()]
    copy_stream = torch.cuda.Stream()
    ev_copy = torch.cuda.Event()
    with torch.cuda.stream(stream):
        sw.run_steps(K, eh, sh, use_graph=True, stream=stream)  # capture
    torch.cuda.synchronize()
    eh.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        sw.run_steps(K, eh, sh, use_graph=True, stream=stream)
    for k in range(K):
        copy_stream.wait_event(events[k])
        with torch.cuda.stream(copy_stream):
            out_e[0].copy_(eh[k], non_blocking=True)
            out_s[0].copy_(sh[k], non_blocking=True)
        ev_copy.record(copy_stream)
        ev_copy.synchronize()
        if k == 0 and not (out_e[0].abs().sum() > 0):
            raise RuntimeError("e2e: step 0's field row reached the host empty")
    e2e_sec = time.perf_counter() - t0
    sw.set_step_events([])
    if not torch.equal(out_e[0], eh[K - 1].cpu()):
        raise RuntimeError("e2e: the host copy of the last step's field differs from the device")
    d2h = out_e[0].numel() * 8 + out_s[0].numel() * 8
    return ms, prof, clk, (e2e_sec, 0, d2h), sw


def single_run_summary(args, name, precision, steps=10, warmup=3):
    """One of the single-run workloads (large: 4096 x 8192 two-stream; driven:
    64 x 1024 with the sin^2 driver) timed as the main bench times its
    workload: CUDA events around a graph of `steps` steps, then three profiled
    steps (kernel times per launch: the call's leading kick, the row passes
    with the next step's leading kick, and the call's last row pass without
    it, apart), then e2e through the C-ABI call with the step's time and
    driver row copied in from pinned host memory and its stored fields and
    series read back, every step."""
    w = WORKLOADS[name]
    sub = argparse.Namespace(steps=steps, warmup=warmup, prof_steps=3, precision=precision)
    ms, prof, clk, e2e, plan = run_gpu(sub, w, 0, 1)
    cells = w["nx"] * w["nv"]
    e2e_sec, h2d, d2h = e2e
    out = {"precision": precision, "ms_per_step": ms / steps, "value": cells * steps / (ms / 1e3),
           "unit": "cell-updates/s",
           "e2e": {"value": cells * steps / e2e_sec, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": d2h},
           "kernels": {k: {"launches": d["launches"], "avg_ms": d["total_ms"] / d["launches"]}
                       for k, d in prof.items()}}
    plan.close()
    if w["kind"] == "driven":
        out["dropin"] = dropin_summary(w, precision)
    return out


def dropin_summary(w, precision, batch=100, calls=100):
    """The single-run workload through the reference-facing Python entry
    points (vlapy/outer_loop.py:248-281 and vlapy/core/step.py:286-328): the
    inner loop over a batch of `batch` steps, with the host time and driver
    arrays copied in and the batch's sim_config brought back to host memory
    as StorageManager.batch_update receives it, and the per-step closure
    timestep(temp_storage, i) called `calls` times.  Wall-clock seconds with
    a device synchronise at both ends, after one untimed call of each."""
    import torch
    from vlapy_gb300 import field_driver, outer_loop, storage
    from vlapy_gb300.core import step
    st = initial_state(w)
    nx = w["nx"]
    pl = pulses_of(w)
    drv = field_driver.PulseDriver(st["x"], {"p": dict(pl[0], envelope="sin2")}) if pl else None
    rules = {"time": "first-last", "space": ["k0", "k1"]}
    stuff = {"nx": nx, "nv": w["nv"], "x": st["x"], "v": st["v"], "kx": st["kx"], "kv": st["kv"],
             "one_over_kx": st["inv"], "dv": st["dv"], "dt": w["dt"], "nu": w["nu"], "driver_function": drv,
             "rules_to_store_f": rules, "f": st["f"], "e": np.zeros(nx)}
    params = {"nu": w["nu"], "fokker-planck": {"type": w["op"], "solver": "batched_tridiagonal"},
              "vlasov-poisson": {"time": "leapfrog", "vdfdx": "exponential", "edfdv": "exponential",
                                 "poisson": "spectral"},
              "backend": {"core": "gb300", "precision": precision}}
    t_host = w["dt"] * np.arange(2 * batch)
    d_host = field_driver.make_driver_array(drv, st["x"], t_host) if drv else np.zeros((2 * batch, nx))
    sc, inner = outer_loop.get_sim_config_and_inner_loop_step(params, stuff, batch, rules)
    sc = inner(t_host[:batch], d_host[:batch], sc)  # captures the batch's graph
    outer_loop.post_inner_loop_update(sc)
    storage.get_batched_data_from_sim_config(sc)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sc = inner(t_host[batch:], d_host[batch:], sc)
    outer_loop.post_inner_loop_update(sc)
    host = storage.get_batched_data_from_sim_config(sc)
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - t0
    h2d = t_host[batch:].nbytes + d_host[batch:].nbytes
    d2h = sum(a.nbytes for a in host[0].values()) + host[1].nbytes + host[2].nbytes + \
        sum(a.nbytes for a in host[3].values()) + host[4].nbytes
    ts = step.get_timestep(params, stuff)
    sc2 = outer_loop.get_arrays_for_inner_loop(stuff, calls + 1, rules)
    sc2["time_batch"] = torch.as_tensor(w["dt"] * np.arange(calls + 1), device="cuda")
    sc2["driver_array_batch"] = torch.as_tensor(
        field_driver.make_driver_array(drv, st["x"], w["dt"] * np.arange(calls + 1)) if drv
        else np.zeros((calls + 1, nx)), device="cuda")
    sc2, _ = ts(sc2, 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(1, calls + 1):
        sc2, _ = ts(sc2, i)
    torch.cuda.synchronize()
    step_s = time.perf_counter() - t0
    return {"inner_loop_ms_per_step": loop_s / batch * 1e3, "inner_loop_batch": batch,
            "inner_loop_h2d_bytes_per_batch": int(h2d), "inner_loop_d2h_bytes_per_batch": int(d2h),
            "timestep_ms_per_call": step_s / calls * 1e3,
            "how": "wall clock: outer_loop inner loop over %d steps (host time/driver arrays in, the sim_config "
                   "to host as batch_update receives it) and %d calls of core.step.get_timestep's closure"
                   % (batch, calls)}


def fp64_plain_sweep(w, steps=2):
    """Plain FP64 GPU method on the whole sweep: every run of the workload in
    one batched FP64 step (vg_batch: the reference's FP64 step per run, the
    parity mode's device code, every launch covering all runs of a shape),
    timed with CUDA events over `steps` steps after one warm-up step and
    extrapolated to the workload's steps per run; then one profiled step."""
    import torch
    from vlapy_gb300.batch import Batch64
    from vlapy_gb300.sweep import sweep_config
    runs = sweep_config(w["n_runs"], w["seed"])
    b = Batch64(runs, vmax=w["vmax"], dt=w["dt"])
    f, e = b.initial_state()
    eh, sh = b.history(steps)
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        b.run_steps(f, e, 1, eh, sh, stream=stream)
        b.run_steps(f, e, steps, eh, sh, use_graph=True, stream=stream)  # capture + first replay
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    with torch.cuda.stream(stream):
        b.run_steps(f, e, steps, eh, sh, use_graph=True, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if not torch.isfinite(eh).all():
        raise RuntimeError("non-finite field in the FP64 batch history")
    b.profile(True)
    with torch.cuda.stream(stream):
        b.run_steps(f, e, 1, eh, sh, stream=stream)
    prof = b.profile_read()
    b.profile(False)
    out = {"runs_per_s": len(runs) / (ms / 1e3 * SWEEP_STEPS), "ms_per_step": ms,
           "cells_per_s": b.cells / (ms / 1e3),
           "kernels_ms_per_step": {k: d["total_ms"] for k, d in prof.items()},
           "how": "all %d runs in one batched FP64 step (vg_batch), %d graph-replayed steps timed with CUDA "
                  "events, extrapolated to %d steps per run" % (len(runs), steps, SWEEP_STEPS)}
    b.close()
    del f, e, eh, sh
    torch.cuda.empty_cache()
    return out


def _damping_errors(t, sw_ref, e_ref, sw, e_hist, t_max=60.0):
    """Relative damping-rate error of each run against the reference runs
    (one peak-envelope fit of |E_1|(t) on [5, t_max] for both)."""
    from vlapy_gb300.diagnostics import damping_fit, mode_amplitude
    out = []
    for i in range(sw.n_runs):
        rf, _ = damping_fit(t, mode_amplitude(sw_ref.e_of(e_ref, i).cpu().numpy()), t_min=5.0, t_max=t_max)
        rg, _ = damping_fit(t, mode_amplitude(sw.e_of(e_hist, i).cpu().numpy()), t_min=5.0, t_max=t_max)
        out.append(abs(rg - rf) / abs(rf) if np.isfinite(rf) and np.isfinite(rg) and rf != 0 else np.nan)
    return np.array(out)


def corrector_training_flops(rows):
    """Tensor-core FLOPs one training step issues on the tcgen05 engine, per
    batch of rows: forward (layer 1: 5 taps x K = 16 at N = 64; layers 2, 3:
    5 taps x K = 64; layer 4: 5 taps x K = 64 at N = 16), data gradients
    (layer 4: K = 16; layers 3, 2: K = 64; all N = 64) and weight gradients
    (M = 128 stacks two taps (one for the input layer's five, padded): 3
    groups x 8 K-steps at N = 16 and N = 64, one group at N = 64)."""
    mma = lambda n, k_steps: 2.0 * 128 * n * 16 * k_steps  # noqa: E731
    fwd = mma(64, 5) + 2 * mma(64, 20) + mma(16, 20)
    dgrad = mma(64, 5) + 2 * mma(64, 20)
    wgrad = mma(16, 24) + 2 * mma(64, 24) + mma(64, 8)
    return rows * (fwd + dgrad + wgrad)


def training_step_timing(cm, data, corr, torch, batch_runs=128, steps=20):
    """ms per Adam step on one batch of batch_runs whole runs (batch_runs x nx
    rows), on each engine, with CUDA events after two untimed steps."""
    x, p, t, f = next(cm._batches(data, batch_runs))
    rows = x.shape[0]
    out = {"rows": rows}
    for engine in ("tcgen05", "mma.sync"):
        c = cm.Corrector(rows, params=corr.params, tau=corr.tau)
        c.set_engine(engine)
        for _ in range(2):
            c.train_step(x, t, p, f, lr=1e-4, group_rows=data.nx)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            c.train_step(x, t, p, f, lr=1e-4, group_rows=data.nx)
        e1.record()
        torch.cuda.synchronize()
        c.check_status()
        ms = e0.elapsed_time(e1) / steps
        out[engine] = {"ms_per_step": ms}
        if engine == "tcgen05":
            out[engine]["tensor_tflops_issued"] = corrector_training_flops(rows) / (ms / 1e3) / 1e12
        c.close()
    return out


def learned_path(args, w):
    """The learned coarse-velocity path (runs of the sweep distribution at
    nx = 64): train the corrector on pairs from fine (nv = 1024) runs, check
    the corrected coarse (nv = 128) runs against the fine runs on held-out
    seeds against fine FP64 runs, and time the corrected coarse step against
    the fine FP32 sweep and the batched FP64 step of the same runs."""
    import torch
    from vlapy_gb300 import corrector as cm
    from vlapy_gb300.sweep import Sweep
    nsteps, nx = SWEEP_STEPS, 64
    t0 = time.perf_counter()
    data = cm.generate_pairs(cm.corrector_runs(args.learned_train, seed=5), n_steps=nsteps)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    n_eval = 256
    t0 = time.perf_counter()
    # three seeds, the best on 64 validation runs (seed 7) kept
    corr, selection = cm.train_selected(data, cm.corrector_runs(64, seed=7), seeds=(0, 1, 2), epochs=4,
                                        max_rows=max(128, n_eval) * nx)
    tau = corr.tau
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    train_step = training_step_timing(cm, data, corr, torch)
    del data
    held = cm.generate_pairs(cm.corrector_runs(n_eval, seed=6), n_steps=nsteps)
    zero = cm.Corrector(128 * nx, params=np.zeros(corr.n_params, np.float32), tau=tau)
    base_loss = cm.evaluate(zero, held)  # zero output: the uncorrected coarse step
    zero.close()
    loss = cm.evaluate(corr, held)
    del held
    # held-out rollouts: fine FP64 (the reference solution: the batched FP64
    # step, the reference's arithmetic), fine FP32 sweep, coarse, corrected coarse
    from vlapy_gb300.batch import Batch64
    ev = cm.corrector_runs(n_eval, seed=6)
    ref64 = Batch64([dict(r, nv=1024) for r in ev], vmax=w["vmax"], dt=w["dt"])
    fj, ej = ref64.initial_state()
    eh64, sh64 = ref64.history(nsteps)
    chunk = 100
    t64 = time.perf_counter()
    for c0 in range(0, nsteps, chunk):
        ref64.run_steps(fj, ej, min(chunk, nsteps - c0), eh64, sh64, row0=c0)
    torch.cuda.synchronize()
    fp64_eval_s = time.perf_counter() - t64
    del fj, ej
    fine, coarse, corrected = (Sweep([dict(r, nv=nv) for r in ev]) for nv in (1024, cm.NV, cm.NV))
    hists = []
    for sw in (fine, coarse):
        sw.reset()
        eh, sh = sw.history(nsteps)
        sw.run_steps(nsteps, eh, sh)
        hists.append((eh, sh))
    corrected.reset()
    ek, sk = corrected.history(nsteps)
    cm.run_corrected(corrected, corr, nsteps, ek, sk)
    torch.cuda.synchronize()
    t = w["dt"] * np.arange(1, nsteps + 1)
    dr_f = _damping_errors(t, ref64, eh64, fine, hists[0][0])
    dr_c = _damping_errors(t, ref64, eh64, coarse, hists[1][0])
    dr_k = _damping_errors(t, ref64, eh64, corrected, ek)
    # mean e^2 per run and step; the batch's series rows are in its stored order
    e2_64 = sh64[:, torch.as_tensor(ref64.slot, device=sh64.device), 3].cpu().numpy()
    e2 = [h[1][:, :, 3].cpu().numpy() for h in hists] + [sk[:, :, 3].cpu().numpy()]
    e2_err = [np.linalg.norm(e - e2_64, axis=0) / np.linalg.norm(e2_64, axis=0) for e in e2]
    ref64.close()
    del eh64, sh64

    def stats(a):
        a = a[np.isfinite(a)]
        return {"median": float(np.median(a)), "max": float(a.max()), "frac_within_1pct": float(np.mean(a <= 0.01)),
                "n": int(a.size)}

    # throughput on 2048 runs: corrected coarse step vs fine FP32 sweep step
    runs = cm.corrector_runs(2048, seed=7)
    K = max(5, min(args.steps, 20))
    out = {}
    for name, nv in (("learned", cm.NV), ("fine_fp32", 1024)):
        sw = Sweep([dict(r, nv=nv) for r in runs])
        sw.reset()
        big = cm.Corrector(sw.cells // cm.NV, params=corr.params, tau=tau) if name == "learned" else None
        step = (lambda n: cm.run_corrected(sw, big, n)) if big else (lambda n: sw.run_steps(n))
        step(3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        step(K)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / K
        out[name] = {"ms_per_step": ms, "runs_per_s": len(runs) / (ms / 1e3 * nsteps)}
        if big:
            # tensor roofline of the network alone: forward FLOPs of one apply over its time
            g = sw.state_view().view(-1, cm.NV)
            rows = g.shape[0]
            flops = corrector_issued_flops(rows, cm.NV)
            prev = g.clone()
            e0.record()
            for _ in range(K):
                big.apply(g, prev, None, out=prev, group_rows=nx)
            e1.record()
            torch.cuda.synchronize()
            ams = e0.elapsed_time(e1) / K
            pk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"] if os.path.exists(
                os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
            out[name]["corrector_ms"] = ams
            out[name]["tensor_roofline"] = {"bound": "tensor", "achieved": flops / (ams / 1e3) / 1e12, "peak": pk,
                                            "unit": "TFLOP/s", "frac": flops / (ams / 1e3) / 1e12 / pk,
                                            "flops_per_apply": flops,
                                            "note": "fused tcgen05 forward (BF16, FP32 accumulate in TMEM) + "
                                                    "projection; padded channels counted as issued"}
            big.close()
        sw.close()
    # plain FP64 GPU method on the same 2048 runs: the batched FP64 step
    b64 = Batch64([dict(r, nv=1024) for r in runs], vmax=w["vmax"], dt=w["dt"])
    fb, eb = b64.initial_state()
    b64.run_steps(fb, eb, 1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b64.run_steps(fb, eb, 3)
    e1.record()
    torch.cuda.synchronize()
    fp64_ms = e0.elapsed_time(e1) / 3
    b64.close()
    del fb, eb
    out["plain_fp64_batched"] = {"ms_per_step": fp64_ms, "runs_per_s": len(runs) / (fp64_ms / 1e3 * nsteps)}
    return {
        "workload": "%d training runs (seed 5), 64 validation runs (seed 7) choosing among 3 trained seeds, "
                    "%d held-out runs (seed 6) of the sweep distribution at nx=64; fine nv=1024, coarse nv=128, "
                    "vmax=6.4, dt=0.1, %d steps" % (args.learned_train, n_eval, nsteps),
        "pairs_s": gen_s, "train_s": train_s, "train_step": train_step, "model_selection": selection, "tau": tau,
        "heldout_one_step_loss": {"uncorrected": base_loss, "corrected": loss, "ratio": loss / base_loss},
        "damping_rate_rel_err_vs_fine_fp64": {"fine_fp32": stats(dr_f), "coarse": stats(dr_c),
                                               "corrected": stats(dr_k)},
        "field_energy_history_rel_err_vs_fine_fp64": {"fine_fp32": stats(e2_err[0]), "coarse": stats(e2_err[1]),
                                                      "corrected": stats(e2_err[2])},
        "throughput_2048_runs": out,
        "reference_solution": "fine (nv = 1024) runs of the batched FP64 step (vg_batch: the reference's FP64 arithmetic), "
                 "%d runs x %d steps in %.1f s" % (n_eval, nsteps, fp64_eval_s),
    }


def main_corrector(args, w, rank, world):
    """Time one correction (vg_corr_apply) of every row of 2048 coarse runs
    (nx = 64, nv = 128): seeded synthetic rows and seeded network weights,
    on the fused tcgen05 kernel (the default engine)."""
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the corrector has no reference counterpart"}))
        return
    import torch
    from vlapy_gb300 import corrector as cm
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)) % max(1, torch.cuda.device_count()))
    nx, runs = w["nx"], w["n_runs"]
    rows = runs * nx
    rng = np.random.default_rng(11)
    p = cm.init_params(3)
    p[-(5 * 64 + 1):-1] = rng.uniform(-0.1, 0.1, 5 * 64).astype(np.float32)  # a live last layer
    v = -w["vmax"] + 2 * w["vmax"] / cm.NV * (np.arange(cm.NV) + 0.5)
    base = np.exp(-v ** 2 / 2)[None, :]
    g = torch.as_tensor((1e-3 * base * rng.standard_normal((rows, cm.NV))).astype(np.float32), device="cuda")
    prev = (g * 0.99).contiguous()
    feat = torch.full((rows,), 0.5, dtype=torch.float32, device="cuda")
    corr = cm.Corrector(rows, params=p, tau=0.02)
    out = torch.empty_like(g)
    K, W = args.steps, args.warmup
    for _ in range(W):
        corr.apply(g, prev, feat, out=out, group_rows=nx)
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(K):
        corr.apply(g, prev, feat, out=out, group_rows=nx)
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    corr.check_status()
    ms = e0.elapsed_time(e1) / K
    # end to end: host rows in pinned memory, copied in and the corrected rows copied back
    hg = g.cpu().pin_memory()
    hp = prev.cpu().pin_memory()
    ho = torch.empty_like(hg).pin_memory()
    dg, dp = torch.empty_like(g), torch.empty_like(prev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        dg.copy_(hg, non_blocking=True)
        dp.copy_(hp, non_blocking=True)
        corr.apply(dg, dp, feat, out=out, group_rows=nx)
        ho.copy_(out, non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / K
    flops = corrector_issued_flops(rows, cm.NV)
    pk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"] if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
    if rank != 0:
        return
    tf = flops / (ms / 1e3) / 1e12
    line = {"metric": "corrected rows/s", "value": rows / (ms / 1e3), "unit": "rows/s", "n_gpus": 1, "steps": K,
            "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "corrector", "rows": rows, "nv": cm.NV, "layers": "4 x conv1d k=5, 64 ch",
                       "engine": "tcgen05 fused forward + projected, capped correction",
                       "l2": "rows %.0f MB in, %.0f MB out: larger than L2 (129 MB)" % (rows * 512 * 2 / 1e6,
                                                                                      rows * 512 / 1e6)},
            "roofline": {"bound": "tensor", "achieved": tf, "peak": pk, "unit": "TFLOP/s", "frac": tf / pk,
                         "traffic": None, "peak_source": "measured" if pk != 1900.0 else "fallback",
                         "flops_per_launch": flops,
                         "note": "issued MMA FLOPs (layer 1 taps folded into K, 20 -> 32; layer 4 taps in N, 5 -> 16)"},
            "e2e": {"value": rows / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": 2 * rows * cm.NV * 4,
                    "d2h_bytes_per_step": rows * cm.NV * 4},
            "gpu_launches": 4 * K, "clocks": clk, "cpu_baseline": None}
    print(json.dumps(line))


def main_corrector_train(args, w, rank, world):
    """Time one training step (vg_corr_train_step: forward layers, projected
    loss, data and weight gradients, Adam, weight packing) of the corrector on
    a batch of 128 runs x 64 rows (seeded synthetic rows, targets and
    weights), on the tcgen05 engine and, for comparison, on mma.sync."""
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the corrector has no reference counterpart"}))
        return
    import torch
    from vlapy_gb300 import corrector as cm
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)) % max(1, torch.cuda.device_count()))
    nx, runs = w["nx"], w["n_runs"]
    rows = runs * nx
    rng = np.random.default_rng(12)
    v = -w["vmax"] + 2 * w["vmax"] / cm.NV * (np.arange(cm.NV) + 0.5)
    base = np.exp(-v ** 2 / 2)[None, :]
    g = torch.as_tensor((1e-3 * base * rng.standard_normal((rows, cm.NV))).astype(np.float32), device="cuda")
    prev = (g * 0.99).contiguous()
    target = (g + 1e-5 * torch.as_tensor(rng.standard_normal((rows, cm.NV)).astype(np.float32), device="cuda"))
    feat = torch.full((rows,), 0.5, dtype=torch.float32, device="cuda")
    K, W = args.steps, args.warmup
    out = {}
    clk = None
    for engine in ("tcgen05", "mma.sync"):
        corr = cm.Corrector(rows, params=cm.init_params(3), tau=0.02)
        corr.set_engine(engine)
        for _ in range(W):
            corr.train_step(g, target, prev, feat, lr=1e-4, group_rows=nx)
        torch.cuda.synchronize()
        if engine == "tcgen05":
            clocks = ClockSampler(torch.cuda.current_device())
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(K):
            corr.train_step(g, target, prev, feat, lr=1e-4, group_rows=nx)
        e1.record()
        torch.cuda.synchronize()
        if engine == "tcgen05":
            clk = clocks.stop()
        corr.check_status()
        out[engine] = e0.elapsed_time(e1) / K
        corr.close()
    if rank != 0:
        return
    ms = out["tcgen05"]
    flops = corrector_training_flops(rows)
    pk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"] if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
    tf = flops / (ms / 1e3) / 1e12
    line = {"metric": "trained rows/s", "value": rows / (ms / 1e3), "unit": "rows/s", "n_gpus": 1, "steps": K,
            "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "corrector-train", "rows": rows, "nv": cm.NV,
                       "engine": "tcgen05 per-layer forward, data- and weight-gradient kernels"},
            "mma_sync_ms_per_step": out["mma.sync"],
            "roofline": {"bound": "tensor", "achieved": tf, "peak": pk, "unit": "TFLOP/s", "frac": tf / pk,
                         "traffic": None, "peak_source": "measured" if pk != 1900.0 else "fallback",
                         "flops_per_step": flops,
                         "note": "issued MMA FLOPs of the nine layer kernels; they are bound by their activation "
                                 "traffic in HBM, not by the MMAs"},
            "e2e": None, "gpu_launches": None, "clocks": clk, "cpu_baseline": None}
    print(json.dumps(line))


def _oracle_sweep_sample(args):
    """One pool task: oracle steps of one sampled sweep run (host cores)."""
    r, steps, vmax, dt = args
    import numpy as np
    from oracle import vlapy_oracle as vo
    nx, nv, k = r["nx"], r["nv"], r["k"]
    run = vo.OracleRun(nx, nv, 2 * np.pi / k, vmax, dt, nu=r["nu"], operator="dg", n_modes=2)
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / k, nx)
    f = vo.maxwellian(nx, nv, vmax) * (1.0 + r["amplitude"] * np.cos(k * x))[:, None]
    st = vo.new_storage(f, np.zeros(nx), steps, 2)
    st["time_batch"] = dt * np.arange(steps)
    st["driver_array_batch"] = np.zeros((steps, nx))
    t0 = time.perf_counter()
    for i in range(steps):
        run.timestep(st, i)
    return nx * nv * steps, time.perf_counter() - t0


def cpu_baseline_sweep(w, n_sample=36, steps=10, cores=None, reps=1, warmup=0):
    """Reference step (CPU oracle) on a stratified sample of sweep runs, one
    process per host core; aggregate cell-updates/s and extrapolated runs/s.
    One sample advances every sampled run by `steps` oracle steps; `warmup`
    untimed samples run first, then `reps` timed ones."""
    import multiprocessing as mp
    from vlapy_gb300.sweep import sweep_config
    runs = sweep_config(w["n_runs"], w["seed"])
    classes = {}
    for r in runs:
        classes.setdefault((r["nx"], r["nv"]), []).append(r)
    per_class = max(1, n_sample // len(classes))
    sample = []
    for key in sorted(classes):
        sample += classes[key][:per_class]
    cores = cores or os.cpu_count() or 1
    walls, results = [], []
    with mp.get_context("spawn").Pool(min(cores, len(sample))) as pool:
        # warm the workers (imports, first FFT plans) before timing
        pool.map(_oracle_sweep_sample, [(r, 1, w["vmax"], w["dt"]) for r in sample])
        for _ in range(warmup):
            pool.map(_oracle_sweep_sample, [(r, steps, w["vmax"], w["dt"]) for r in sample])
        for _ in range(max(1, reps)):
            t0 = time.perf_counter()
            results.append(pool.map(_oracle_sweep_sample, [(r, steps, w["vmax"], w["dt"]) for r in sample]))
            walls.append(time.perf_counter() - t0)
    cells = sum(c for res in results for c, _ in res)
    # seconds per step per class (single core), then the whole sweep on `cores` cores
    sec_class = {}
    for res in results:
        for r, (c, sec) in zip(sample, res):
            sec_class.setdefault((r["nx"], r["nv"]), []).append(sec / steps)
    core_sec = sum(np.mean(sec_class[key]) * len(classes[key]) for key in classes) * SWEEP_STEPS
    runs_per_s = len(runs) / (core_sec / min(cores, len(sample)))
    wall = sum(walls)
    value = cells / wall
    return value, runs_per_s, min(cores, len(sample)), len(sample), steps, wall


def cpu_baseline(w, steps, reps_cap=3):
    """Oracle (NumPy restatement of the reference step) on the host cores."""
    from oracle import vlapy_oracle as vo
    st = initial_state(w)
    nx, nv = w["nx"], w["nv"]
    pl = pulses_of(w)
    drv = None
    if pl:
        p = pl[0]
        drv = lambda t: vo.driver_sin2(st["x"], p["k0"], p["w0"], p["a0"], p["t_R"], t)  # noqa: E731
    run = vo.OracleRun(nx, nv, 2 * np.pi / w["k"], w["vmax"], w["dt"], nu=w["nu"], operator=w["op"],
                       driver=drv, n_modes=2)
    n = max(1, min(steps, reps_cap))
    stg = vo.new_storage(st["f"], np.zeros(nx), n, 2)
    stg["time_batch"] = w["dt"] * np.arange(n)
    stg["driver_array_batch"] = np.zeros((n, nx))
    t0 = time.perf_counter()
    for i in range(n):
        run.timestep(stg, i)
    dt = time.perf_counter() - t0
    return nx * nv * n / dt, n, dt


def main_fp64sweep(args, w, rank, world):
    """The batched FP64 step on the sweep's runs (the plain FP64 GPU method)
    as its own workload: K graph-replayed steps timed with CUDA events after
    one untimed step, then one profiled step.  The default workload reports
    the same measurement as fp64_plain_gpu; this one exists to profile the
    FP64 kernels alone."""
    import torch
    from vlapy_gb300 import _lib
    if rank != 0:
        return
    _lib.load()
    out = fp64_plain_sweep(w, steps=args.steps)
    cells = out["cells_per_s"] * out["ms_per_step"] / 1e3
    line = {"metric": "cell-updates/s", "value": out["cells_per_s"], "unit": "cell-updates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": 1, "ms_per_step": out["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "fp64sweep", "n_runs": w["n_runs"], "seed": w["seed"], "cells": cells},
            "runs_per_s": out["runs_per_s"], "kernels_ms_per_step": out["kernels_ms_per_step"]}
    print(json.dumps(line))
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sweep", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32-deltaf"])
    ap.add_argument("--prof-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--runs", type=int, default=None, help="sweep size (default: the 4096-run workload)")
    ap.add_argument("--no-fp64-compare", action="store_true", help="skip the plain FP64 GPU sweep estimate")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned coarse-velocity path")
    ap.add_argument("--learned-train", type=int, default=2048, help="fine training runs of the learned path")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    w = dict(WORKLOADS[args.workload])
    if args.runs:
        w["n_runs"] = args.runs
    if w["kind"] == "sweep":
        return main_sweep(args, w, rank, world)
    if w["kind"] == "corrector":
        return main_corrector(args, w, rank, world)
    if w["kind"] == "corrector-train":
        return main_corrector_train(args, w, rank, world)
    if w["kind"] == "fp64sweep":
        return main_fp64sweep(args, w, rank, world)
    cells = w["nx"] * w["nv"]
    metric = "cell-updates/s"
    cfg = {"workload": args.workload, "nx": w["nx"], "nv": w["nv"], "dt": w["dt"], "nu": w["nu"],
           "collision": w["op"] if w["nu"] > 0 else "none", "integrator": "leapfrog",
           "precision": args.precision, "storage": "fields+series+k0,k1 modes every step",
           "l2": "state (%.0f MB) %s L2 (129 MB)" % (cells * (8 if args.precision == "fp64" else 4) / 1e6,
                                                   "larger than" if cells * (8 if args.precision == "fp64" else 4) > 129e6
                                                   else "smaller than")}

    if args.impl == "reference":
        if rank != 0:
            return
        val, n, sec = cpu_baseline(w, args.steps)
        line = {"metric": metric, "value": val, "unit": "cell-updates/s", "n_gpus": args.gpus,
                "steps": n, "warmup": 0, "ms_per_step": 1e3 * sec / n, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": cfg, "impl": "reference",
                "cpu_baseline": {"value": val, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                                 "sample": "%d full oracle step(s) of the workload" % n},
                "e2e": {"value": val, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    from vlapy_gb300 import replicas
    replicas.init(world)
    ms, prof, clk, e2e, plan = run_gpu(args, w, int(os.environ.get("LOCAL_RANK", rank)), world)
    # replicas: every rank advances its own copy of the run
    t_max, _, value = replicas.aggregate(ms, cells * args.steps, world)
    e2e_sec, h2d, d2h = e2e
    _, _, e2e_val = replicas.aggregate(1e3 * e2e_sec, cells * args.steps, world)
    dom = max(prof.items(), key=lambda kv: kv[1]["total_ms"])
    name, pd = dom
    avg_ms = pd["total_ms"] / pd["launches"]
    peak, peak_kind = peaks()
    achieved = pd["bytes_per_launch"] / (avg_ms / 1e3) / 1e9
    launches_per_step = 0
    kernels_per_launch = {"storage": 3, "field_f32": 2, "store_f32": 2}
    for k, d in prof.items():
        per = d["launches"] / args.prof_steps
        launches_per_step += per * kernels_per_launch.get(k, 1)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        cval, n, sec = cpu_baseline(w, args.steps, reps_cap=1)
        cpu = {"value": cval, "unit": "cell-updates/s", "cores": 1, "kind": "port",
               "sample": "%d full oracle step (VP+FP+storage) of the %dx%d workload, %.1f s" % (n, w["nx"], w["nv"], sec)}
    line = {
        "metric": metric, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
        "data": "synthetic", "config": cfg,
        "e2e": {"value": e2e_val, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "kernel": name,
                     "peak_source": peak_kind,
                     "kernel_ms": avg_ms, "bytes_per_launch": pd["bytes_per_launch"]},
        "kernels": {k: {"launches": d["launches"], "avg_ms": d["total_ms"] / d["launches"]} for k, d in prof.items()},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))


def main_sweep(args, w, rank, world):
    cfg = {"workload": "sweep", "n_runs": w["n_runs"], "seed": w["seed"], "nx": [32, 64, 128],
           "nv": [256, 512, 1024], "vmax": w["vmax"], "dt": w["dt"], "collision": "dg (25% of runs nu=0)",
           "integrator": "leapfrog", "precision": "fp32-deltaf (FP64 moment/zero-mode reductions)",
           "storage": "per run and step: field e[nx] + 7 series", "run_steps": SWEEP_STEPS}
    if args.impl == "reference":
        if rank != 0:
            return
        # each bench step: the 36 stratified runs advanced 36 oracle steps (~1 s
        # on 16 cores), W untimed then K timed
        val, rps, cores, n, osteps, wall = cpu_baseline_sweep(w, n_sample=36, steps=36, reps=args.steps,
                                                              warmup=args.warmup)
        line = {"metric": "cell-updates/s", "value": val, "unit": "cell-updates/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(1, args.steps),
                "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg, "impl": "reference",
                "runs_per_s": rps,
                "cpu_baseline": {"value": val, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                                 "sample": "each step: %d sweep runs (stratified over the 9 shapes) x %d full "
                                           "oracle steps, one process per core; %d timed steps, %.1f s wall; "
                                           "runs/s extrapolated to 4096 runs x 2000 steps"
                                           % (n, osteps, args.steps, wall)},
                "e2e": {"value": val, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    from vlapy_gb300 import replicas
    replicas.init(world)
    ms, prof, clk, e2e, sw = run_sweep_gpu(args, w, int(os.environ.get("LOCAL_RANK", rank)), world, rank)
    cells = sw.cells
    tma_flags, tma = sw.status()
    # every rank advances its own shard: units summed, time the slowest rank's
    t_max, total_cells, value = replicas.aggregate(ms, cells * args.steps, world)
    runs_per_s = world * sw.n_runs / (t_max / args.steps / 1e3 * SWEEP_STEPS)
    e2e_sec, h2d, d2h = e2e
    _, _, e2e_value = replicas.aggregate(1e3 * e2e_sec, cells * args.steps, world)
    dom_name, dom = max(prof.items(), key=lambda kv: kv[1]["total_ms"])
    avg_ms = dom["total_ms"] / dom["launches"]
    peak, peak_kind = peaks()
    achieved = dom["bytes_per_launch"] / (avg_ms / 1e3) / 1e9
    # kernel launches in the timed graph of K steps: per step one x-drift
    # launch per nx class, the field solve, one row-pass launch per nv class
    # and the store; per call one kick-only launch per nv class
    n_x = len({r["nx"] for r in sw.runs})
    n_v = len({r["nv"] for r in sw.runs})
    timed_launches = args.steps * (n_x + 1 + n_v + 1) + n_v
    if rank != 0:
        return
    fp64 = None
    if not args.no_fp64_compare:
        fp64 = fp64_plain_sweep(w)
    learned = None if args.no_learned else learned_path(args, w)
    singles = None
    if not args.no_fp64_compare:
        import torch
        singles = {}
        for name, prec, k in (("large", "fp32-deltaf", 20), ("large", "fp64", 3), ("driven", "fp32-deltaf", 50),
                              ("driven", "fp64", 20)):
            singles["%s_%s" % (name, prec)] = single_run_summary(args, name, prec, steps=k)
            torch.cuda.empty_cache()
    cpu = None
    if not args.no_cpu_baseline:
        cval, crps, cores, n, steps, wall = cpu_baseline_sweep(w, n_sample=36, steps=360)
        cpu = {"value": cval, "unit": "cell-updates/s", "cores": cores, "kind": "port", "runs_per_s": crps,
               "sample": "%d sweep runs (stratified over the 9 shapes) x %d full oracle steps, one process per "
                         "core, %.1f s wall" % (n, steps, wall)}
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
        "runs_per_s": runs_per_s,
        "fp64_plain_gpu": fp64,
        "single_runs": singles,
        "x_drift_tma": tma,
        "learned_path": learned,
        "e2e": {"value": e2e_value, "unit": "cell-updates/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": ROW_PASS_DRAM_BYTES_PER_CELL * cells if dom_name == "sweep_row_pass" else None,
                     "traffic_source": "ncu dram bytes of the three full row-pass launches of the 4096-run sweep, "
                                       "per cell; below the algorithmic 8 B/cell because some written rows stay in L2 "
                                       "past the launch",
                     "kernel": dom_name, "peak_source": peak_kind, "kernel_ms": avg_ms,
                     "bytes_per_launch": dom["bytes_per_launch"]},
        "kernels": {k: {"launches": d["launches"], "avg_ms": d["total_ms"] / d["launches"]} for k, d in prof.items()},
        "gpu_launches": timed_launches,
        "clocks": clk,
        "cpu_baseline": cpu,
        "state_bytes": cells * 4,
        "l2": "state %.0f MB, larger than L2 (129 MB)" % (cells * 4 / 1e6),
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()

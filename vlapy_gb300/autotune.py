"""Autotuner of the batched sweep's kernel shapes.

The sweep kernels (csrc/vg_sweep.cu) take their per-shape choices from
build-time constants: the FFT radix of each nv class of the row pass and of
each nx class of the x-drift (bit masks over log2 of the size), the threads
of a row-kernel CTA, and the resident CTAs per SM each kernel is compiled for
(its register budget per thread).  ``tune`` searches them on the GPU it runs
on, one constant at a time from the current values (coordinate descent).  For
each candidate value it

1. builds the library with it into a scratch folder (only vg_sweep.cu is
   recompiled);
2. in a fresh process, advances a sweep of the given runs from its initial
   state and compares the stored fields with those of the starting build.
   A different radix rounds differently, so the comparison is a relative L2
   bound, not bit equality.  A candidate that fails to build, to run or to
   match is dropped;
3. times the sweep step there: CUDA events around a CUDA graph of K steps
   after W warm-up steps, the best of three repeats;
4. keeps the value when it is faster than the current best by more than the
   noise margin.

``--write`` stores the winners in vlapy_gb300/tuning.json, which the build
passes to nvcc as -D definitions.  The candidates of each constant are the
values its kernels are written for and were measured with: radix masks over
the size classes each radix supports (radix 32 for nv >= 256, radix 16 for
nv >= 64 and 32 <= nx <= 256), 256-, 128- or 64-thread row CTAs, and 2 to 4
resident CTAs per SM.

Usage (on a GPU machine; each candidate costs one build and one short run):

    python -m vlapy_gb300.autotune --runs 4096 --steps 20 --warmup 3 --write
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

from . import build as B

# (constant, candidate values); the starting value is taken from the tuning in use
KNOBS = (
    ("VG_SWEEP_R32_MASK", (0x600, 0x400, 0x0, 0x700)),  # radix 32 for nv = 512 and 1024, 1024 only, none, or 256 up
    ("VG_SWEEP_R16_MASK", (0x700, 0x500, 0x300)),    # radix 16 for nv in {256, 512, 1024}, or a subset
    ("VG_ROW_MIN_BLOCKS_R16", (3, 2, 4)),            # row CTAs per SM of the radix-16 classes
    ("VG_SWEEP_ROW_BLOCK", (256, 128, 64)),          # threads of a row-kernel CTA
    ("VG_SWEEP_COL_R16_MASK", (0xE0, 0xC0, 0x80, 0x0)),  # radix 16 for the x-drift of nx = 32 up, 64 up, 128 only, or none
    ("VG_COL_MIN_BLOCKS_R16", (3, 2)),               # x-drift CTAs per SM of the radix-16 classes
    ("VG_SWEEP_COL_R32_MASK", (0x0, 0x80, 0xC0)),    # radix 32 for the x-drift: none, nx = 128, or nx = 64 and 128
)

MATCH_TOL = 1e-4  # relative L2 of the stored fields against the starting build


class CandidateError(RuntimeError):
    """A candidate that did not build, run or match."""


def coordinate_search(knobs, start, measure, margin=0.01, log=None):
    """Coordinate descent over the knobs from `start`.

    measure(values) returns the step time (ms) of a configuration or raises
    CandidateError.  A value replaces the current best when its time is below
    (1 - margin) x the best time.  Returns (best values, best ms, records),
    records being (name, value, ms or None, error text or None) per trial."""
    best = dict(start)
    best_ms = measure(best)
    records = [("start", None, best_ms, None)]
    for name, candidates in knobs:
        for val in candidates:
            if best.get(name) == val:
                continue
            trial = dict(best)
            trial[name] = val
            try:
                ms = measure(trial)
            except CandidateError as err:
                records.append((name, val, None, str(err)))
                if log:
                    log("%s=%d: dropped (%s)" % (name, val, (str(err).splitlines() or [""])[0][:120]))
                continue
            records.append((name, val, ms, None))
            if log:
                log("%s=%d: %.4f ms/step (best %.4f)" % (name, val, ms, best_ms))
            if ms < (1.0 - margin) * best_ms:
                best, best_ms = trial, ms
    return best, best_ms, records


def relative_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


class Measurer:
    """Builds candidate libraries into a scratch folder and times each in a
    fresh process (a process loads one library); the first measured
    configuration is the reference its successors must match."""

    def __init__(self, n_runs, seed, steps, warmup, workdir, python=sys.executable):
        self.n_runs, self.seed, self.steps, self.warmup = n_runs, seed, steps, warmup
        self.workdir = workdir
        self.python = python
        self.reference = None
        self.count = 0

    def __call__(self, values):
        self.count += 1
        lib = os.path.join(self.workdir, "lib%d" % self.count, "libvlagpu.so")
        try:
            B.build(tuning=values, lib_path=lib, build_dir=os.path.join(self.workdir, "objs"))
        except RuntimeError as err:
            raise CandidateError("build failed: %s" % err) from None
        out = os.path.join(self.workdir, "probe%d.npz" % self.count)
        cmd = [self.python, "-m", "vlapy_gb300.autotune", "probe", "--lib", lib, "--runs", str(self.n_runs),
               "--seed", str(self.seed), "--steps", str(self.steps), "--warmup", str(self.warmup), "--out", out]
        r = subprocess.run(cmd, capture_output=True, text=True, cwd=B.ROOT)
        if r.returncode != 0:
            raise CandidateError("probe failed (exit %d): %s" % (r.returncode, r.stderr[-2000:]))
        d = np.load(out)
        fields = d["e"]
        if not np.isfinite(fields).all():
            raise CandidateError("non-finite fields")
        if self.reference is None:
            self.reference = fields
        else:
            err = relative_l2(fields, self.reference)
            if not err <= MATCH_TOL:
                raise CandidateError("fields differ from the starting build by %.3e" % err)
        return float(d["ms"])


def probe(lib, n_runs, seed, steps, warmup, out, repeats=3):
    """Time one library (run in a fresh process): the sweep step in ms, best of
    `repeats` graph replays of `steps` steps, and the fields stored by the
    first replay (after `warmup` steps from the initial state)."""
    from . import _lib
    _lib.load(lib)
    import torch

    from .sweep import Sweep, sweep_config

    sw = Sweep(sweep_config(n_runs, seed))
    eh, sh = sw.history(steps)
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        sw.reset(stream)
        sw.run_steps(warmup, use_graph=False, stream=stream)
        sw.run_steps(steps, eh, sh, use_graph=True, stream=stream)  # capture (and one run)
        sw.reset(stream)
        sw.run_steps(warmup, use_graph=False, stream=stream)
    torch.cuda.synchronize()
    best = None
    fields = None
    for rep in range(repeats):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        with torch.cuda.stream(stream):
            sw.run_steps(steps, eh, sh, use_graph=True, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        best = ms if best is None else min(best, ms)
        if rep == 0:
            fields = eh.cpu().numpy()
    np.savez(out, ms=np.float64(best), e=fields)


def tune(n_runs=4096, seed=20261203, steps=20, warmup=3, margin=0.01, write=False, log=print):
    """Search the knobs on this machine's GPU; returns (values, ms, records)."""
    start = dict(B.read_tuning())
    for name, candidates in KNOBS:
        start.setdefault(name, candidates[0])
    with tempfile.TemporaryDirectory(prefix="vg_autotune_") as work:
        meas = Measurer(n_runs, seed, steps, warmup, work)
        best, best_ms, records = coordinate_search(KNOBS, start, meas, margin=margin, log=log)
    if write:
        write_tuning(best, best_ms, records, n_runs, seed, steps)
    return best, best_ms, records


def write_tuning(values, ms, records, n_runs, seed, steps, path=B.TUNING_FILE):
    """Store the tuned constants (and what they were measured on)."""
    gpu = "unknown GPU"
    try:
        import torch
        gpu = torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001 - the name is only a label
        pass
    doc = {
        "source": "autotune",
        "note": "Measured by vlapy_gb300.autotune on %s, %s: sweep of %d runs (seed %d), %d steps a replay; "
                "%.4f ms per step." % (gpu, time.strftime("%Y-%m-%d"), n_runs, seed, steps, ms),
        "values": {k: int(v) for k, v in values.items()},
        "trials": [{"name": n, "value": v, "ms": m, "error": e} for n, v, m, e in records],
    }
    B.tuning_flags(doc["values"])  # refuse anything the build would refuse
    with open(path, "w") as fh:
        json.dump(doc, fh, indent=2)
        fh.write("\n")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd")
    pp = sub.add_parser("probe", help="time one built library (internal: one process per candidate)")
    pp.add_argument("--lib", required=True)
    pp.add_argument("--out", required=True)
    for p in (ap, pp):
        p.add_argument("--runs", type=int, default=4096)
        p.add_argument("--seed", type=int, default=20261203)
        p.add_argument("--steps", type=int, default=20)
        p.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--margin", type=float, default=0.01, help="relative gain a change must bring")
    ap.add_argument("--write", action="store_true", help="store the result in vlapy_gb300/tuning.json")
    args = ap.parse_args(argv)
    if args.cmd == "probe":
        probe(args.lib, args.runs, args.seed, args.steps, args.warmup, args.out)
        return
    best, ms, _ = tune(args.runs, args.seed, args.steps, args.warmup, args.margin, args.write)
    print(json.dumps({"values": best, "ms_per_step": ms}))


if __name__ == "__main__":
    main()

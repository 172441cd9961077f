"""Build libvlagpu.so (the C-ABI CUDA library) in-tree with nvcc for sm_103a.

Each translation unit under ``csrc/`` is compiled in parallel to an object
file, then linked into ``vlapy_gb300/_lib/libvlagpu.so``.  Host code is
compiled with ``-ffp-contract=off`` so that host-side coefficient arithmetic
(integrator sub-steps) rounds exactly like the reference's Python floats on
both x86-64 and aarch64.

The batched sweep's kernel shapes (FFT radix per size class, CTA size,
resident CTAs per SM) are build-time constants of ``csrc/vg_sweep.cu``.
``tuning.json`` beside this file (written by ``vlapy_gb300.autotune``) holds
their values; they reach nvcc as ``-D`` definitions for that file.  An object
is rebuilt when its sources or its compile flags change.
"""

from __future__ import annotations

import concurrent.futures as cf
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvlagpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

TUNING_FILE = os.path.join(HERE, "tuning.json")
# the build-time constants a tuning may set, and the translation unit that reads them
TUNABLE = ("VG_SWEEP_R32_MASK", "VG_SWEEP_R16_MASK", "VG_ROW_MIN_BLOCKS_R16", "VG_ROW_MIN_BLOCKS_R32",
           "VG_ROW_MIN_BLOCKS", "VG_SWEEP_ROW_BLOCK", "VG_SWEEP_COL_R16_MASK", "VG_COL_MIN_BLOCKS_R16",
           "VG_COL_MIN_BLOCKS", "VG_KICK_MIN_BLOCKS", "VG_SWEEP_COL_R32_MASK", "VG_COL_MIN_BLOCKS_R32")
TUNED_SOURCE = "vg_sweep.cu"


def read_tuning(path: str = TUNING_FILE) -> dict:
    """The tuned constants of a tuning file ({} when there is none)."""
    if not os.path.exists(path):
        return {}
    with open(path) as fh:
        return dict(json.load(fh).get("values", {}))


def tuning_flags(values: dict) -> list:
    """-D definitions of tuned constants; only the names in TUNABLE, integer values."""
    flags = []
    for name in sorted(values):
        val = values[name]
        if name not in TUNABLE:
            raise ValueError("not a tunable build constant: %r" % (name,))
        if isinstance(val, bool) or not isinstance(val, int) or val < 0:
            raise ValueError("%s must be a non-negative integer, got %r" % (name, val))
        flags.append("-D%s=%d" % (name, val))
    return flags


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvlagpu.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(nvcc, src, obj, extra):
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           "-I", CSRC, "-c", src, "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (os.path.basename(src), r.stdout, r.stderr))
    return r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _stamp(obj):
    return obj + ".flags"


def _flags_changed(obj, flags):
    """True when obj was compiled with other flags than these (or has no record)."""
    try:
        with open(_stamp(obj)) as fh:
            return fh.read() != " ".join(flags)
    except OSError:
        return True


def build(force: bool = False, verbose: bool = False, extra=(), tuning=None, lib_path=None,
          build_dir=None) -> str:
    """Compile (if needed) and return the path of libvlagpu.so.

    tuning: the sweep's tuned constants (default: those of tuning.json);
    lib_path / build_dir: where the library and the objects go (default: the
    in-tree library and build folder)."""
    nvcc = nvcc_path()
    lib_path = lib_path or LIB
    build_dir = build_dir or BUILD_DIR
    tuned = tuning_flags(read_tuning() if tuning is None else tuning)
    os.makedirs(os.path.dirname(lib_path), exist_ok=True)
    os.makedirs(build_dir, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(ROOT, "include", "vlagpu.h"))
    objs = [os.path.join(build_dir, os.path.basename(s)[:-3] + ".o") for s in srcs]
    flags = {s: [*extra, *(tuned if os.path.basename(s) == TUNED_SOURCE else [])] for s in srcs}
    todo = [(s, o) for s, o in zip(srcs, objs)
            if force or _stale(o, [s, *headers]) or _flags_changed(o, flags[s])]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            futs = {ex.submit(_compile, nvcc, s, o, flags[s]): (s, o) for s, o in todo}
            for fut in cf.as_completed(futs):
                msg = fut.result()
                s, o = futs[fut]
                with open(_stamp(o), "w") as fh:
                    fh.write(" ".join(flags[s]))
                if verbose and msg:
                    sys.stderr.write(msg)
    if force or todo or _stale(lib_path, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", lib_path, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return lib_path


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(force="--force" in sys.argv, verbose=v or bool(extra), extra=extra))

"""Host logic of the sweep autotuner and of the tuned build (no GPU): the
tuning file, the -D definitions it becomes, the per-object flag records that
trigger rebuilds, and the coordinate search over a synthetic cost."""

import json
import os
import re

import pytest

from vlapy_gb300 import autotune as AT
from vlapy_gb300 import build as B


def _source_defaults():
    src = open(os.path.join(B.CSRC, B.TUNED_SOURCE)).read()
    found = {}
    for name, val in re.findall(r"#ifndef (VG_\w+)\s*\n#define \1 (\w+)", src):
        found[name] = int(val, 0)
    return found


def test_committed_tuning_reproduces_the_source_defaults():
    """The committed tuning names only constants of vg_sweep.cu; while it is the
    'defaults' tuning, its values are the source's own, so the tuned build is
    the build the GPU tests and profiles ran."""
    defaults = _source_defaults()
    assert set(B.TUNABLE) <= set(defaults)
    doc = json.load(open(B.TUNING_FILE))
    assert set(doc["values"]) <= set(B.TUNABLE)
    if doc["source"] == "defaults":
        assert doc["values"] == {k: defaults[k] for k in doc["values"]}
    B.tuning_flags(doc["values"])


def test_tuning_flags_are_whitelisted_integers():
    assert B.tuning_flags({"VG_SWEEP_R16_MASK": 0x700, "VG_ROW_MIN_BLOCKS_R16": 3}) == [
        "-DVG_ROW_MIN_BLOCKS_R16=3", "-DVG_SWEEP_R16_MASK=1792"]
    with pytest.raises(ValueError):
        B.tuning_flags({"VG_PAD_SHIFT_F32": 3})      # not a sweep knob
    with pytest.raises(ValueError):
        B.tuning_flags({"VG_SWEEP_ROW_BLOCK": "256 -DX=1"})
    with pytest.raises(ValueError):
        B.tuning_flags({"VG_SWEEP_ROW_BLOCK": -1})
    assert B.tuning_flags({}) == []


def test_knob_candidates_are_buildable_values():
    defaults = _source_defaults()
    for name, cands in AT.KNOBS:
        assert name in B.TUNABLE
        assert cands[0] == defaults[name]            # the search starts from the source default
        assert len(set(cands)) == len(cands)
        B.tuning_flags({name: c for c in cands[:1]})
        for c in cands:
            B.tuning_flags({name: c})


def test_flag_records_trigger_rebuilds(tmp_path):
    obj = str(tmp_path / "vg_sweep.o")
    assert B._flags_changed(obj, ["-DVG_SWEEP_R16_MASK=1792"])   # no record yet
    with open(B._stamp(obj), "w") as fh:
        fh.write(" ".join(["-DVG_SWEEP_R16_MASK=1792"]))
    assert not B._flags_changed(obj, ["-DVG_SWEEP_R16_MASK=1792"])
    assert B._flags_changed(obj, ["-DVG_SWEEP_R16_MASK=1280"])
    assert B._flags_changed(obj, [])


def test_read_tuning_missing_file_is_empty(tmp_path):
    assert B.read_tuning(str(tmp_path / "none.json")) == {}


def test_coordinate_search_on_a_synthetic_cost():
    knobs = (("A", (1, 2, 3)), ("B", (10, 20)), ("C", (0, 1)))
    cost = {("A", 1): 0.0, ("A", 2): -0.3, ("A", 3): -0.1, ("B", 10): 0.0, ("B", 20): -0.005,
            ("C", 0): 0.0, ("C", 1): 0.0}
    calls = []

    def measure(v):
        calls.append(dict(v))
        if v["C"] == 1:
            raise AT.CandidateError("fields differ")
        return 1.0 + sum(cost[(k, v[k])] for k in ("A", "B", "C"))

    best, ms, records = AT.coordinate_search(knobs, {"A": 1, "B": 10, "C": 0}, measure, margin=0.01)
    assert best == {"A": 2, "B": 10, "C": 0}          # B=20 gains under the 1 % margin
    assert ms == pytest.approx(0.7)
    assert calls[0] == {"A": 1, "B": 10, "C": 0}
    assert ("C", 1, None, "fields differ") in records
    assert len(calls) == 1 + 2 + 1 + 1                # start, A=2, A=3, B=20, C=1


def test_write_tuning_round_trip(tmp_path):
    path = str(tmp_path / "tuning.json")
    vals = {"VG_SWEEP_R32_MASK": 0, "VG_SWEEP_ROW_BLOCK": 128}
    AT.write_tuning(vals, 1.5, [("start", None, 1.6, None), ("VG_SWEEP_R32_MASK", 0, 1.5, None)],
                    4096, 1, 20, path=path)
    doc = json.load(open(path))
    assert doc["source"] == "autotune"
    assert B.read_tuning(path) == vals
    assert doc["trials"][1] == {"name": "VG_SWEEP_R32_MASK", "value": 0, "ms": 1.5, "error": None}
    with pytest.raises(ValueError):
        AT.write_tuning({"NOT_A_KNOB": 1}, 1.0, [], 1, 1, 1, path=path)


def test_relative_l2():
    assert AT.relative_l2([1.0, 2.0], [1.0, 2.0]) == 0.0
    assert AT.relative_l2([0.0], [0.0]) == 0.0
    assert AT.relative_l2([1.0, 0.0], [0.0, 1.0]) == pytest.approx(2 ** 0.5)


def test_measurer_orchestration(tmp_path, monkeypatch):
    """Measurer with the build stubbed and a stand-in interpreter for the probe
    process: the first configuration becomes the reference, a candidate whose
    fields differ, whose probe fails or whose build fails is dropped, and a
    matching one returns its time."""
    import stat
    import sys

    import numpy as np

    builds = []

    def fake_build(tuning=None, lib_path=None, build_dir=None, **kw):
        if tuning.get("VG_SWEEP_ROW_BLOCK") == 64:
            raise RuntimeError("nvcc failed")
        os.makedirs(os.path.dirname(lib_path), exist_ok=True)
        open(lib_path, "w").write(json.dumps(tuning))     # the probe reads the tuning back
        builds.append(dict(tuning))
        return lib_path

    monkeypatch.setattr(AT.B, "build", fake_build)
    probe = tmp_path / "fake_python"
    probe.write_text(
        "#!%s\n"
        "import json, sys, numpy as np\n"
        "a = sys.argv[1:]\n"
        "tuning = json.load(open(a[a.index('--lib') + 1]))\n"
        "if tuning.get('VG_COL_MIN_BLOCKS_R16') == 2: sys.exit(3)\n"
        "e = np.ones((4, 8)) * (1.5 if tuning.get('VG_SWEEP_R32_MASK') == 0 else 1.0)\n"
        "np.savez(a[a.index('--out') + 1], ms=np.float64(2.0 - tuning.get('VG_ROW_MIN_BLOCKS_R16', 3) / 10), e=e)\n"
        % sys.executable)
    probe.chmod(probe.stat().st_mode | stat.S_IEXEC)
    meas = AT.Measurer(16, 1, 4, 3, str(tmp_path), python=str(probe))
    base = {"VG_SWEEP_R32_MASK": 0x400, "VG_ROW_MIN_BLOCKS_R16": 3, "VG_COL_MIN_BLOCKS_R16": 3,
            "VG_SWEEP_ROW_BLOCK": 256}
    assert meas(base) == pytest.approx(1.7)
    assert meas(dict(base, VG_ROW_MIN_BLOCKS_R16=4)) == pytest.approx(1.6)
    with pytest.raises(AT.CandidateError, match="differ"):
        meas(dict(base, VG_SWEEP_R32_MASK=0))
    with pytest.raises(AT.CandidateError, match="probe failed"):
        meas(dict(base, VG_COL_MIN_BLOCKS_R16=2))
    with pytest.raises(AT.CandidateError, match="build failed"):
        meas(dict(base, VG_SWEEP_ROW_BLOCK=64))
    assert len(builds) == 4

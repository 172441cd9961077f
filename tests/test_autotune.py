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

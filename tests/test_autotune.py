"""The autotuner's host logic without a GPU: the library's knobs, the cache, and the choice of
each knob's fastest value (timings stubbed)."""
from __future__ import annotations

import importlib
import json

import pytest


@pytest.fixture()
def tune(ss, native):
    mod = importlib.import_module("sphere-stereo_gb300.autotune")
    saved = {k: mod.get(k) for k in mod.KNOBS}
    yield mod
    for k, v in saved.items():
        mod.set_knob(k, v)


def test_knobs_and_choices(tune):
    assert tune.choices("sweep_variant") == [0, 1, 2, 3]
    assert tune.choices("hole_blocks_per_sm") == [2, 4, 8]
    assert tune.choices("merge_frames") == [2, 4, 8]
    assert tune.choices("uneven_span") == [1, 2, 4]
    assert tune.choices("isb_up_blocks") == [2, 3]
    assert tune.choices("isb_select_blocks") == [2, 3]
    assert tune.choices("isb_tile_tma") == [0, 1]
    assert tune.choices("hole_persistent") == [0, 1]
    assert tune.choices("sweep_tiles") == [0, 16, 32]
    assert tune.choices("hole_tail") == [0, 3, 4, 6, 8]
    assert tune.choices("select_whole") == [0, 1]
    assert tune.choices("up_whole") == [0, 1]
    assert tune.choices("isb_tail") == [0, 256, 1024, 4096]
    assert tune.choices("post_tail") == [0, 1024, 4096, 16384]
    assert tune.choices("stage_columns") == [0, 1]
    tune.set_knob("merge_frames", 8)
    assert tune.get("merge_frames") == 8
    with pytest.raises(ValueError):
        tune.set_knob("merge_frames", 3)
    assert tune.get("merge_frames") == 8


def test_cache_round_trip_and_apply(tune, tmp_path):
    path = tmp_path / "tuning.json"
    path.write_text(json.dumps({"k": {"sweep_variant": 2, "merge_frames": 2, "unknown": 5}}))
    t = tune.Tuner(str(path))
    assert t.apply("missing") is None
    assert t.apply("k") == {"sweep_variant": 2, "merge_frames": 2}
    assert tune.get("sweep_variant") == 2 and tune.get("merge_frames") == 2
    # caller choices (not library knobs) are kept in the cache and returned
    path.write_text(json.dumps({"k": {"sweep_variant": 1, "overlap_groups": 2}}))
    t = tune.Tuner(str(path))
    assert t.apply("k") == {"sweep_variant": 1, "overlap_groups": 2}
    assert tune.get("sweep_variant") == 1


def test_tune_picks_the_fastest_choice(tune, tmp_path, monkeypatch):
    # fake timings: the entry's time depends on the knob value that is set when it runs
    cost = {"sweep_variant": {0: 3.0, 1: 1.0, 2: 2.0, 3: 2.5}, "merge_frames": {2: 5.0, 4: 4.0, 8: 6.0}}
    runs = []

    class FakeTimer:
        def __init__(self, entries):
            self.entry = entries
            self.events = []

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            pass

        def total_ms(self):
            name = next(n for n, (_, e) in tune.KNOBS.items() if e == self.entry)
            return cost[name][tune.get(name)] * len(self.events)

    def run():
        runs.append(1)
        if FakeTimer.current is not None:
            FakeTimer.current.events.append(None)

    FakeTimer.current = None

    class Recording(FakeTimer):
        def __enter__(self):
            FakeTimer.current = self
            return self

        def __exit__(self, *exc):
            FakeTimer.current = None

    monkeypatch.setattr(tune, "_EntryTimer", Recording)
    path = tmp_path / "t.json"
    t = tune.Tuner(str(path))
    best = t.tune("w", run, ["sweep_variant", "merge_frames"], repeats=2)
    assert best == {"sweep_variant": 1, "merge_frames": 4}
    assert tune.get("sweep_variant") == 1 and tune.get("merge_frames") == 4
    assert len(runs) == (4 + 3) * (1 + 2)  # every choice of both knobs: one warm-up and two timed runs
    assert json.loads(path.read_text())["w"] == best
    assert tune.Tuner(str(path)).apply("w") == best


def test_workload_key_is_bounded(tune):
    k = tune.workload_key("uneven", [((512, 512), 32, 4, 2)] * 200)
    assert len(k) < 400 and "sha1:" in k
    assert tune.workload_key("uneven", [((512, 512), 32, 4, 2)] * 200) == k

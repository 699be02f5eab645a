"""Autotuner of the batched kernels' launch shapes (no counterpart in the reference).

The library exposes a few launch-shape knobs (include/sphere_stereo_gb300.h, SSG_TUNE_*): the
sweep's block shape, the blocks per SM of the hole-filling steps, the frames one merge thread
handles, the work-item span of the uneven sweep and the register bounds of the ISB upsampling
(coarse levels and the fused selecting level).  For a workload (a key naming the device and
the shapes), ``Tuner.tune`` runs the caller's launch sequence eagerly, times the entry point each
knob affects with CUDA events on the stream it is enqueued on, one knob at a time over its
choices (coordinate descent: the knobs act on different kernels), and keeps the fastest.  Results
are cached in a JSON file so that later runs of the same workload skip the search.

Knob values are process-wide and read when a launch is enqueued: a caller sets its values
(``Tuner.apply``) before launching or capturing a CUDA graph, and the graph keeps them.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
from typing import Callable

import torch

from . import _native as N

# knob name -> (SSG_TUNE_* id, the entry points whose kernels it shapes)
KNOBS = {
    "sweep_variant": (N.TUNE_SWEEP_VARIANT, ("ssg_sweep_cost_batch", "ssg_sweep_cost_batch_entries")),
    "hole_blocks_per_sm": (N.TUNE_HOLE_BLOCKS_PER_SM, ("ssg_inpaint_holes_batch",)),
    "merge_frames": (N.TUNE_MERGE_FRAMES, ("ssg_merge_panorama_batch_approx",)),
    "uneven_span": (N.TUNE_UNEVEN_SPAN, ("ssg_uneven_run",)),
    "isb_up_blocks": (N.TUNE_ISB_UP_BLOCKS, ("ssg_isb_upsample_batch", "ssg_isb_filter_batch")),
    "isb_select_blocks": (N.TUNE_ISB_SELECT_BLOCKS, ("ssg_isb_upsample_select_batch",)),
    "isb_tile_tma": (N.TUNE_ISB_TILE_TMA, ("ssg_isb_upsample_batch", "ssg_isb_filter_batch",
                                           "ssg_isb_upsample_select_batch")),
    "hole_persistent": (N.TUNE_HOLE_PERSISTENT, ("ssg_inpaint_holes_batch",)),
    "sweep_tiles": (N.TUNE_SWEEP_TILES, ("ssg_sweep_cost_batch", "ssg_sweep_cost_batch_entries")),
    "hole_tail": (N.TUNE_HOLE_TAIL, ("ssg_inpaint_holes_batch",)),
    "select_whole": (N.TUNE_SELECT_WHOLE, ("ssg_isb_upsample_select_batch",)),
    "up_whole": (N.TUNE_UP_WHOLE, ("ssg_isb_upsample_batch", "ssg_isb_filter_batch")),
    "isb_tail": (N.TUNE_ISB_TAIL, ("ssg_isb_filter_batch",)),
    "post_tail": (N.TUNE_POST_TAIL, ("ssg_isb_apply_batch",)),
    "stage_columns": (N.TUNE_STAGE_COLUMNS, ("ssg_stage_images", "ssg_stage_images_u8", "ssg_stage_images_resized")),
}


# choices made by the caller rather than the library (name -> meaning), cached with the knobs
CHOICES = {
    "overlap_groups": "frame groups of a batch whose post-filter and stitch overlap the next group's sweep",
}


def default_cache_path() -> str:
    env = os.environ.get("SSG_TUNING_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "sphere_stereo_gb300", "tuning.json")


def choices(knob: str) -> list[int]:
    kid = KNOBS[knob][0]
    buf = (ctypes.c_int32 * 16)()
    n = N.library().ssg_tuning_choices(kid, buf, 16)
    return [int(buf[i]) for i in range(n)]


def get(knob: str) -> int:
    return int(N.library().ssg_tuning_get(KNOBS[knob][0]))


def set_knob(knob: str, value: int) -> None:
    N.call("ssg_tuning_set", KNOBS[knob][0], int(value))


class _EntryTimer:
    """Brackets every call of the given entry points with CUDA events on the stream it is
    launched on."""

    def __init__(self, entries: tuple[str, ...]):
        self.entries = entries
        self.events = []
        self._orig = None

    def __enter__(self):
        self._orig = N.call
        orig, entries, events = self._orig, self.entries, self.events

        def call(name, *args):
            if name not in entries:
                return orig(name, *args)
            stream = torch.cuda.ExternalStream(args[-1]) if args[-1] else torch.cuda.current_stream()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            orig(name, *args)
            b.record(stream)
            events.append((a, b))

        N.call = call
        return self

    def __exit__(self, *exc):
        N.call = self._orig

    def total_ms(self) -> float:
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in self.events)


class Tuner:
    def __init__(self, cache_path: str | None = None):
        self.cache_path = default_cache_path() if cache_path is None else cache_path
        self.cache: dict[str, dict[str, int]] = {}
        try:
            with open(self.cache_path) as f:
                data = json.load(f)
            if isinstance(data, dict):
                self.cache = {k: {n: int(v) for n, v in d.items() if n in KNOBS or n in CHOICES}
                              for k, d in data.items() if isinstance(d, dict)}
        except (OSError, ValueError):
            pass

    def _save(self) -> None:
        try:
            os.makedirs(os.path.dirname(self.cache_path) or ".", exist_ok=True)
            tmp = f"{self.cache_path}.{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump(self.cache, f, indent=1, sort_keys=True)
            os.replace(tmp, self.cache_path)
        except OSError:
            pass  # a read-only home keeps the results in memory only

    def apply(self, key: str) -> dict[str, int] | None:
        """Sets the knobs cached for ``key``; returns them (with the cached caller choices), or None
        when the key is not cached."""
        values = self.cache.get(key)
        if values is None:
            return None
        for name, v in values.items():
            if name in KNOBS:
                set_knob(name, v)
        return dict(values)

    def pick(self, key: str, name: str, runs: dict, stream: int, repeats: int = 3) -> int:
        """Times each whole launch sequence of ``runs`` (choice -> eager launches on ``stream``)
        with CUDA events on that stream, caches the fastest choice as ``name`` for ``key`` and
        returns it."""
        s = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
        timings = {}
        for value, run in runs.items():
            run()  # warm-up
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            for _ in range(repeats):
                run()
            b.record(s)
            b.synchronize()
            timings[value] = a.elapsed_time(b) / repeats
        best = min(timings, key=timings.get)
        self.cache.setdefault(key, {})[name] = int(best)
        self._save()
        return int(best)

    def tune(self, key: str, run: Callable[[], None], knobs: list[str], repeats: int = 3,
             entry: str | None = None) -> dict[str, int]:
        """Picks each knob's fastest choice for the launch sequence ``run`` (eager launches on the
        current stream), timing the entry points the knob shapes (or ``entry`` for every knob),
        sets it, caches and returns the choices."""
        best: dict[str, int] = {}
        for name in knobs:
            entries = (entry,) if entry else KNOBS[name][1]
            before = get(name)
            timings = {}
            for value in choices(name):
                set_knob(name, value)
                run()  # warm-up with this shape (first-use set-up, caches)
                with _EntryTimer(entries) as t:
                    for _ in range(repeats):
                        run()
                if t.events:
                    timings[value] = t.total_ms() / repeats
            if timings:
                best[name] = min(timings, key=timings.get)
                set_knob(name, best[name])
            else:  # the sequence never called the knob's entry points: leave it as it was
                set_knob(name, before)
        self.cache[key] = best
        self._save()
        return best


def workload_key(*parts) -> str:
    """A cache key: the device's name and the shapes that select the kernels' work (long shape
    lists are kept as a digest)."""
    name = torch.cuda.get_device_name(torch.cuda.current_device()) if torch.cuda.is_available() else "cpu"
    text = "|".join(str(p) for p in parts)
    if len(text) > 200:
        text = text[:80] + "|sha1:" + hashlib.sha1(text.encode()).hexdigest()
    return f"{name}|{text}"

"""Benchmark: RGB-D panoramas per second at 1024 x 1024 matching, 32 candidates (the synthetic
stand-in for the reference's prototype configuration: 4 double-sphere fisheye cameras, inputs
1216 x 1216, references 2 and 3, rgb_to_stitch 1216 x 1216, panorama 2048 x 1024, sigma_i 10,
sigma_s 25, min/max distance 0.55 / 100 m).

One step = one batch of B RGB-D panoramas (distance estimation on both reference cameras +
stitching, for B frames) through RGBD_Estimator.estimate_RGBD_panoramas; value = panoramas/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--batch B]

--impl reference times the reference algorithm on the host cores: the C restatement of the
reference (oracle/, OpenMP over all cores), one full frame per step.  Under torchrun only rank 0
runs it.  --gpus N > 1 runs N independent replicas (frames are independent; no collective on
the data path), timed between barriers, max over ranks.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PACKAGE = "sphere-stereo_gb300"

WORKLOAD = dict(width_in=1216, matching=(1024, 1024), stitch=(1216, 1216), panorama=(2048, 1024), candidates=32,
                refs=[2, 3], sigma_i=10.0, sigma_s=25.0, min_dist=0.55, max_dist=100.0)
WORKLOAD_NAME = ("4 double-sphere fisheye cameras (fx=0.28W, xi=-0.2, alpha=0.6) on a 0.2 m square, "
                 "1216x1216 uint8 inputs, matching 1024x1024, 32 candidates, references 2,3, "
                 "rgb_to_stitch 1216x1216, panorama 2048x1024, sigma_i 10, sigma_s 25")
METRIC = "RGB-D panoramas/s @1024² match, 32 cand"
DTYPE = {storage: (f"{storage} level-0 cost storage, f32 coarse levels and arithmetic; the sweep samples the "
                   "resized images in 8.8 fixed point with 16-bit bilinear weights (integer dot products)")
         for storage in ("fp16", "unorm16")}
UNIT = "panoramas/s"
DATA = ("synthetic: seeded 6x5x3 m box room + 20 value-noise spheres, ray-cast per frame (seed 2000+frame) to "
        "1216x1216 uint8 per camera; images to match = those resized to the matching resolution in float32 "
        "(linear, the reference's cv2.resize), images to stitch = the 1216x1216 renders")
# DRAM bytes (read + write) of sweep_batch_kernel per (frame, reference) instance with fp16 storage,
# measured by ncu on one launch of an 8-frame batch of this workload (1,189,412,608 B read +
# 1,038,806,784 B written for 16 instances)
SWEEP_DRAM_BYTES_PER_INSTANCE = (1189412608 + 1038806784) // 16


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def frames_for_rank(total: int, rank: int, world: int) -> list[int]:
    """Frame ids a replica renders for its input pool: disjoint across ranks."""
    return [rank + world * i for i in range(total)]


def render_pool(count: int, rank: int, world: int, resize):
    """Seeded frames of the workload: every camera ray-cast to width_in x width_in uint8 (the
    inputs), the images to match made from them by `resize` (uint8 [cameras, rows, cols, 3],
    (cols, rows) -> float32 [cameras, ...]: the library's GPU resize, or for the reference arm the
    oracle's restatement of the same arithmetic), the images to stitch the renders of the
    references (rgb_to_stitch = the input resolution).  frame.originals keeps the uint8 renders."""
    syn = importlib.import_module(PACKAGE + ".synthetic")
    cams = syn.square_rig(WORKLOAD["width_in"])
    w = WORKLOAD["width_in"]
    if tuple(WORKLOAD["stitch"]) != (w, w):
        raise ValueError("the workload stitches at its input resolution")
    ids = frames_for_rank(max(1, count), rank, world)
    # the ray casting is numpy on the host: frames render in parallel worker processes (spawned,
    # so that no CUDA state is inherited)
    import concurrent.futures
    import multiprocessing

    workers = max(1, min(len(ids), (os.cpu_count() or 1) // 2))
    if workers > 1:
        with concurrent.futures.ProcessPoolExecutor(workers, mp_context=multiprocessing.get_context("spawn")) as pool:
            renders = list(pool.map(render_frame, ids))
    else:
        renders = [render_frame(f) for f in ids]
    frames = []
    for originals, inv in renders:
        match = resize(originals, WORKLOAD["matching"])
        fr = syn.Frame(list(match), [originals[r] for r in WORKLOAD["refs"]], inv)
        fr.originals = originals
        frames.append(fr)
    return syn.basalt_calibration(cams), frames


def render_frame(f: int):
    """Frame f of the workload: every camera ray-cast to width_in x width_in uint8 (seed
    synthetic.frame_seed(2, f)); returns (uint8 [cameras, w, w, 3], ground-truth inverse distances)."""
    syn = importlib.import_module(PACKAGE + ".synthetic")
    w = WORKLOAD["width_in"]
    cams = syn.square_rig(w)
    rng = np.random.Generator(np.random.PCG64(syn.frame_seed(2, f)))
    fr = syn.render_frame(syn.random_scene(rng), cams, (w, w), (w, w), [])
    return np.stack(fr.images_to_match), fr.inv_distance


def gpu_resize(device):
    ss_utils = importlib.import_module(PACKAGE + ".utils")

    def resize(images, size):
        import torch

        return ss_utils.resize_linear(torch.as_tensor(images, device=device), size).cpu().numpy()

    return resize


def oracle_resize(images, size):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import prep_eval_oracle

    return np.stack([prep_eval_oracle.resize_linear(im, size) for im in images])


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> tuple[float, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class LaunchRecorder:
    """Counts this library's kernel launches and brackets one entry point with CUDA events on
    the stream it is launched on."""

    def __init__(self, native, *timed_entries: str):
        self.native = native
        self.timed_entries = timed_entries
        self.launches = 0
        self.events = []
        self.active = False
        self._orig = native.call

    def __enter__(self):
        import torch

        native = self.native

        def call(name, *args):
            if not self.active:
                return self._orig(name, *args)
            self.launches += native.kernels_launched(name, args)
            if name in self.timed_entries:
                stream = torch.cuda.ExternalStream(args[-1]) if args[-1] else torch.cuda.current_stream()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                self._orig(name, *args)
                b.record(stream)
                self.events.append((a, b))
                return None
            return self._orig(name, *args)

        native.call = call
        return self

    def __exit__(self, *exc):
        self.native.call = self._orig

    def mean_ms(self) -> float | None:
        if not self.events:
            return None
        return sum(a.elapsed_time(b) for a, b in self.events) / len(self.events)


def level_pixels(cols: int, rows: int) -> list[int]:
    """Pixels of each ISB level (python/isb_filter.py:59-69): L = int(min(log2 cols, log2 rows) - 1)
    levels of ceil(rows / 2^l) x ceil(cols / 2^l)."""
    import math

    L = int(min(math.log2(cols), math.log2(rows)) - 1)
    return [-(-rows // 2 ** l) * -(-cols // 2 ** l) for l in range(L)]


def sweep_bytes_per_instance(cols: int, rows: int, cameras: int, references: int, candidates: int,
                             cost_bytes: int) -> int:
    """Algorithmic bytes of the sweep for one (frame, reference) instance, by the byte model of the
    hot path: each float32 image to match read once per frame (12 B per pixel and camera, shared
    by the frame's references), the camera-selection map (1 B per pixel) and the cost volume
    written once (cost_bytes x candidates per pixel).  89 B per pixel at 1024^2, 4 cameras, 2
    references, 32 fp16 candidates."""
    P = cols * rows
    return (12 * cameras * P) // references + P + cost_bytes * candidates * P


def frame_bytes(cols: int, rows: int, cameras: int, references: int, candidates: int, cost_bytes: int,
                stitch_pixels: int, panorama_pixels: int) -> int:
    """Algorithmic bytes of one RGB-D panorama, by the same model: float32 inputs read once; per
    reference the cost volume (sweep write, level-0 read by the downsampling, the last upsampling
    read fused with the selection: 3 P; coarse levels written, read and read-modify-written:
    4 sum(P_l)), two guide pyramids of 3 bytes per pixel, the distance post-filter's float32
    pyramid, the distance map; the stitch (16 B per matching pixel and reference, float32 blend
    weights per panorama pixel and reference, 7 B of outputs per panorama pixel).  781 P at
    1024^2 / 32 fp16 candidates / 1216^2 stitch / 2048 x 1024 panorama."""
    levels = level_pixels(cols, rows)
    P, coarse = levels[0], sum(levels[1:])
    b_in = 12 * cameras * P + 12 * references * stitch_pixels
    per_ref = (cost_bytes * candidates * (3 * P + 4 * coarse) + 2 * 3 * (2 * P + 4 * coarse) +
               4 * (3 * P + 4 * coarse) + 4 * P)
    b_stitch = 16 * P * references + 4 * references * panorama_pixels + 7 * panorama_pixels
    return b_in + references * per_ref + b_stitch


def _estimator(ss, calibration, device, storage, batch, graphs, tuner=None, output_slots=1):
    import torch

    W = WORKLOAD
    calibs = ss.parse_json_calib(calibration, W["matching"], device)
    vp = torch.zeros(3, device=device)
    for r in W["refs"]:
        vp += calibs[r].rt[:3, 3] / len(W["refs"])
    mw, mh = W["matching"]
    masks = [torch.ones(1, mh, mw, device=device) for _ in calibs]
    return ss.RGBD_Estimator(calibs, W["min_dist"], W["max_dist"], W["candidates"], W["refs"], vp, masks,
                             W["matching"], W["stitch"], W["panorama"], W["sigma_i"], W["sigma_s"], device,
                             cost_storage=storage, max_batch=batch, cuda_graphs=graphs, tuner=tuner,
                             output_slots=output_slots)


def run_ours(args, rank, world, device, rendered):
    import torch

    ss = importlib.import_module(PACKAGE)
    native = ss._native
    calibration, frames = rendered
    B = args.batch
    autotune = importlib.import_module(PACKAGE + ".autotune")
    tuner = None if args.no_autotune else autotune.Tuner()
    for kv in args.knob:
        name, value = kv.split("=")
        autotune.set_knob(name, int(value))
    est = _estimator(ss, calibration, device, args.storage, B, True, tuner, output_slots=2)
    pipe = est.pipeline()
    if args.overlap_groups is not None:
        pipe.overlap_groups = args.overlap_groups
    mw, mh = WORKLOAD["matching"]

    # two input batches (B frames each, assembled from the rendered frames), device resident:
    # each batch holds B x 83 MB of inputs, far beyond the 126 MB L2, and consecutive steps
    # alternate between them
    def batch_of(k):
        ids = [(k + j) % len(frames) for j in range(B)]
        m = np.stack([np.stack(frames[i].images_to_match) for i in ids]).astype(np.float32)
        st = np.stack([np.stack(frames[i].images_to_stitch) for i in ids]).astype(np.float32)
        return m, st

    host_batches = [batch_of(k) for k in range(2)]
    dev_batches = [(torch.as_tensor(m, device=device), torch.as_tensor(st, device=device)) for m, st in host_batches]
    for i in range(args.warmup):
        est.estimate_RGBD_panoramas(*dev_batches[i % 2])
    torch.cuda.synchronize()
    barrier(world)

    with ClockSampler(device.index) as clocks:
        torch.cuda.synchronize()
        barrier(world)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for i in range(args.steps):
            est.estimate_RGBD_panoramas(*dev_batches[i % 2])
        end.record()
        torch.cuda.synchronize()
        barrier(world)
    ms = max_over_ranks(start.elapsed_time(end) / args.steps, world, device)
    launches = pipe.launches_per_batch(B, float_stitch=True) * args.steps

    # end to end through the public API: pinned host inputs in, panoramas back to pinned host
    # memory, every step.  The next batch's upload runs on an upload stream and the previous
    # batch's download on a download stream, both overlapping the current batch's work: the
    # estimator writes its panoramas to two buffers in turn (output_slots=2), so a batch's are
    # downloaded while the next batch computes into the other buffer.
    pinned = [(torch.as_tensor(m).pin_memory(), torch.as_tensor(st).pin_memory()) for m, st in host_batches]
    staging = [(torch.empty_like(dev_batches[0][0]), torch.empty_like(dev_batches[0][1])) for _ in range(2)]
    out_host = [(torch.empty(pipe.rgb.shape, dtype=torch.uint8).pin_memory(),
                 torch.empty(pipe.pano_distance.shape).pin_memory()) for _ in range(2)]
    h2d = sum(t.numel() * t.element_size() for t in pinned[0])
    d2h = out_host[0][0].numel() + out_host[0][1].numel() * 4
    up_stream, down_stream = torch.cuda.Stream(device), torch.cuda.Stream(device)
    compute = torch.cuda.current_stream(device)
    uploaded = [torch.cuda.Event() for _ in range(2)]
    consumed = [torch.cuda.Event() for _ in range(2)]
    produced = [torch.cuda.Event() for _ in range(2)]
    downloaded = [torch.cuda.Event() for _ in range(2)]

    def upload(i):
        slot = i % 2
        with torch.cuda.stream(up_stream):
            up_stream.wait_event(consumed[slot])
            for d, h in zip(staging[slot], pinned[i % 2]):
                d.copy_(h, non_blocking=True)
            uploaded[slot].record(up_stream)

    def e2e(steps):
        for ev in consumed + downloaded:
            ev.record(compute)
        upload(0)
        for i in range(steps):
            if i + 1 < steps:
                upload(i + 1)
            slot = i % 2
            compute.wait_event(uploaded[slot])
            # the outputs this batch overwrites were those of batch i - 2: downloaded by now
            compute.wait_event(downloaded[slot])
            rgb, dist = est.estimate_RGBD_panoramas(*staging[slot])
            consumed[slot].record(compute)
            produced[slot].record(compute)
            with torch.cuda.stream(down_stream):
                down_stream.wait_event(produced[slot])
                out_host[slot][0].copy_(rgb, non_blocking=True)
                out_host[slot][1].copy_(dist, non_blocking=True)
                downloaded[slot].record(down_stream)
        for ev in downloaded:
            compute.wait_event(ev)  # the timed region ends with every output on the host

    e2e(args.warmup)
    torch.cuda.synchronize()
    barrier(world)
    s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s2.record()
    e2e(args.steps)
    e2.record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(s2.elapsed_time(e2) / args.steps, world, device)

    # dominant kernel: the same steps launched eagerly, CUDA events around its launches
    eager = _estimator(ss, calibration, device, args.storage, B, False)
    rec = LaunchRecorder(native, "ssg_sweep_cost_batch", "ssg_sweep_cost_batch_entries")
    eager.estimate_RGBD_panoramas(*dev_batches[0])
    torch.cuda.synchronize()
    with rec:
        rec.active = True
        for i in range(args.steps):
            eager.estimate_RGBD_panoramas(*dev_batches[i % 2])
        torch.cuda.synchronize()
        rec.active = False
    peak, peak_kind = measured_peaks()
    sweep_ms = rec.mean_ms()
    R = len(WORKLOAD["refs"])
    cost_bytes = 2 if args.storage in ("fp16", "unorm16") else 4
    instances = B * R
    sweep_bytes = instances * sweep_bytes_per_instance(mw, mh, 4, R, WORKLOAD["candidates"], cost_bytes)
    achieved = sweep_bytes / (sweep_ms * 1e-3) / 1e9 if sweep_ms else None
    traffic = (SWEEP_DRAM_BYTES_PER_INSTANCE * instances
               if SWEEP_DRAM_BYTES_PER_INSTANCE is not None and args.storage == "fp16" else None)
    sw, sh = WORKLOAD["stitch"]
    pw, ph = WORKLOAD["panorama"]
    per_frame = frame_bytes(mw, mh, 4, R, WORKLOAD["candidates"], cost_bytes, sw * sh, pw * ph)
    frame_gbs = per_frame * B / (ms * 1e-3) / 1e9

    # the same batches from the 8-bit renders themselves (the decoded images, the reference's
    # per-frame input): their upload, the resize to the matching resolution on the GPU (inside the
    # staging pass, ssg_stage_images_resized), and the references' decoded images stitched from the
    # same upload (the stitch resolution is the decoded one); uploads and downloads overlapped as
    # above
    e2e_u8 = None
    device_u8 = None
    if not args.no_u8:
        originals = [np.stack([frames[(k + j) % len(frames)].originals for j in range(B)]) for k in range(2)]
        pinned_u8 = [torch.as_tensor(o).pin_memory() for o in originals]
        slots_u8 = [torch.empty_like(pinned_u8[0], device=device) for _ in range(2)]
        h2d_u8 = pinned_u8[0].numel()

        # device-resident decoded inputs (2 alternating batches of B x 4 x 4.4 MB, beyond L2): the
        # step includes the resize; information beside `value`, whose inputs are already resized
        resident_u8 = [torch.as_tensor(o, device=device) for o in originals]
        for i in range(args.warmup):
            est.estimate_RGBD_panoramas(resident_u8[i % 2])
        torch.cuda.synchronize()
        barrier(world)
        s4, e4 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s4.record()
        for i in range(args.steps):
            est.estimate_RGBD_panoramas(resident_u8[i % 2])
        e4.record()
        torch.cuda.synchronize()
        u8_dev_ms = max_over_ranks(s4.elapsed_time(e4) / args.steps, world, device)
        device_u8 = {"value": world * B * 1000.0 / u8_dev_ms, "unit": UNIT, "ms_per_step": u8_dev_ms,
                     "inputs": "device-resident decoded 1216x1216 uint8 images of every camera, resized to the "
                               "matching resolution inside the staging pass; the references' images stitched "
                               "from them"}
        del resident_u8

        def upload_u8(i):
            slot = i % 2
            with torch.cuda.stream(up_stream):
                up_stream.wait_event(consumed[slot])
                slots_u8[slot].copy_(pinned_u8[i % 2], non_blocking=True)
                uploaded[slot].record(up_stream)

        def e2e_u8_steps(steps):
            for ev in consumed + downloaded:
                ev.record(compute)
            upload_u8(0)
            for i in range(steps):
                if i + 1 < steps:
                    upload_u8(i + 1)
                slot = i % 2
                compute.wait_event(uploaded[slot])
                compute.wait_event(downloaded[slot])  # the outputs of batch i - 2 are on the host
                rgb, dist = est.estimate_RGBD_panoramas(slots_u8[slot])
                consumed[slot].record(compute)
                produced[slot].record(compute)
                with torch.cuda.stream(down_stream):
                    down_stream.wait_event(produced[slot])
                    out_host[slot][0].copy_(rgb, non_blocking=True)
                    out_host[slot][1].copy_(dist, non_blocking=True)
                    downloaded[slot].record(down_stream)
            for ev in downloaded:
                compute.wait_event(ev)

        e2e_u8_steps(args.warmup)
        torch.cuda.synchronize()
        barrier(world)
        s3, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s3.record()
        e2e_u8_steps(args.steps)
        e3.record()
        torch.cuda.synchronize()
        u8_ms = max_over_ranks(s3.elapsed_time(e3) / args.steps, world, device)
        e2e_u8 = {"value": world * B * 1000.0 / u8_ms, "unit": UNIT, "h2d_bytes_per_step": h2d_u8,
                  "d2h_bytes_per_step": d2h, "ms_per_step": u8_ms,
                  "inputs": "the decoded 1216x1216 uint8 images of every camera (the reference's per-frame input, "
                            "python/main.py:73-81), resized to the matching resolution on the GPU inside the timed "
                            "region (in the staging pass); the references' decoded images stitched from the same "
                            "upload"}
    e2e_f32 = {"value": world * B * 1000.0 / e2e_ms, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
               "inputs": "the float32 images estimate_RGBD_panorama takes (already resized on the host)"}
    return {
        "value": world * B * 1000.0 / ms,
        "ms_per_step": ms,
        # the headline end-to-end number starts where the reference's frame loop starts: decoded
        # 8-bit images on the host
        "e2e": e2e_u8 if e2e_u8 is not None else e2e_f32,
        "e2e_f32": e2e_f32,
        "device_from_decoded_u8": device_u8,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "roofline": {"bound": "hbm", "kernel": "sweep_batch_kernel", "achieved": achieved, "peak": peak,
                     "peak_kind": f"{peak_kind} hbm_gbs (burst copy)", "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this "
                                       "batch, profiles/sweep_batch_kernel_1024_n32.md",
                     "algorithmic_bytes_per_launch": sweep_bytes,
                     "algorithmic_bytes_model": "per instance: 12 B x cameras / references (float32 images to "
                                                "match, once per frame) + 1 B selection + cost_bytes x candidates "
                                                "per pixel",
                     "traffic_over_algorithmic": (traffic / sweep_bytes) if traffic else None,
                     "dram_gbs": (traffic / (sweep_ms * 1e-3) / 1e9) if traffic and sweep_ms else None,
                     "mean_launch_ms": sweep_ms, "launches_timed": len(rec.events),
                     "frame": {"algorithmic_bytes_per_frame": per_frame, "achieved": frame_gbs,
                               "frac": frame_gbs / peak, "unit": "GB/s",
                               "model": "float32 inputs once, per reference the cost pyramid (3 P + 4 sum P_l "
                                        "cells), two guide pyramids, the distance post-filter and map, the "
                                        "stitch tables and outputs"}},
        "tuned": pipe.tuned if pipe.tuned is not None else {k: autotune.get(k) for k in pipe.TUNED_KNOBS},
        "overlap_groups": pipe._group_count(B),
    }


def run_plain_fp32(args, device, rendered, frames_timed: int):
    """The plain fp32 path on the same GPU: one frame per call of estimate_RGBD_panorama, float32
    cost volume, the reference's arithmetic bit for bit (no batching, no CUDA graph)."""
    import torch

    ss = importlib.import_module(PACKAGE)
    calibration, frames = rendered
    est = _estimator(ss, calibration, device, "fp32", 1, False)
    inputs = [([torch.as_tensor(im.astype(np.float32), device=device) for im in f.images_to_match],
               [torch.as_tensor(im.astype(np.float32), device=device) for im in f.images_to_stitch]) for f in frames]
    for i in range(args.warmup):
        est.estimate_RGBD_panorama(*inputs[i % len(inputs)])
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for i in range(frames_timed):
        est.estimate_RGBD_panorama(*inputs[i % len(inputs)])
    end.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / frames_timed
    return {"value": 1000.0 / ms, "unit": UNIT, "ms_per_frame": ms, "frames": frames_timed,
            "mode": "fp32 cost volume, one frame per estimate_RGBD_panorama call, eager launches"}


def run_torch_sweep_gpu(args, device, rendered, frames_timed: int):
    """The reference's torch part restated on the same GPU (python/depth_estimation.py:137-242):
    the sweep over materialised [N, H, W, 3] point volumes with a 5-D grid_sample per camera and
    the torch selection (min / max / gather / parabola); the ISB filter and the stitcher are this
    library's fp32 kernels (the reference's kernels need CuPy, which is not on the GPU host).  An
    informational leg: the target ratio is against the plain fp32 path."""
    import torch

    ss = importlib.import_module(PACKAGE)
    utils = importlib.import_module(PACKAGE + ".utils")
    calibration, frames = rendered
    W = WORKLOAD
    est = _estimator(ss, calibration, device, "fp32", 1, False)
    cols, rows = W["matching"]
    N = W["candidates"]
    calibs = est.calibrations
    yy, xx = torch.meshgrid(torch.arange(rows, device=device), torch.arange(cols, device=device), indexing="ij")
    pixels = torch.stack([xx, yy], dim=-1).unsqueeze(0)
    cands = 1 / torch.linspace(1 / W["min_dist"], 1 / W["max_dist"], N, device=device)
    size = torch.tensor([cols, rows], device=device)

    def distance_of(ref, selected, images_p, image_list):
        pt_unit, _ = utils.unproject(pixels, calibs[ref])
        points = cands.view(N, 1, 1, 1) * pt_unit.view(1, rows, cols, 3)
        volume = torch.zeros([1, 3, N, rows, cols], device=device)
        for c, cal in enumerate(calibs):
            rt = torch.matmul(torch.inverse(cal.rt), calibs[ref].rt)
            in_cam = torch.matmul(torch.cat([points, torch.ones_like(points[..., :1])], dim=-1), rt.T)
            uv, _ = utils.project(in_cam[..., :3], cal)
            uv = ((uv + 0.5) / size) * 2 - 1
            uv = torch.cat([uv.unsqueeze(0), torch.zeros_like(uv[..., :1]).unsqueeze(0)], dim=-1)
            sampled = torch.nn.functional.grid_sample(images_p[c], uv, align_corners=False)
            mask = (selected == c).repeat(1, 3, N, 1, 1)
            volume[mask] = sampled[mask]
        cost = torch.clamp(torch.sum(torch.abs(volume - images_p[ref]), dim=1).squeeze(0), max=500)
        guide = utils.rgb2yCbCr(image_list[ref]).type(torch.uint8)
        cost, _ = est.cost_filter.apply(guide.clone(), cost.clone(), W["sigma_i"], W["sigma_s"])
        m, idx = torch.min(cost, dim=0, keepdim=True)
        M, _ = torch.max(cost, dim=0, keepdim=True)
        left = torch.gather(cost, 0, torch.clamp(idx - 1, 0, N - 1))
        right = torch.gather(cost, 0, torch.clamp(idx + 1, 0, N - 1))
        var = torch.clamp(0.5 * (left - right) / ((left + right) - 2.0 * m + 1e-8), -0.5, 0.5)
        var[idx == N - 1] = 0
        var[idx == 0] = 0
        sel = idx.float() + var
        sel[M == m] = N - 1
        dist = cands[0] / ((cands[0] / cands[-1] - 1) * sel / (N - 1) + 1)
        dist[torch.abs(M - m) < 1e-8] = cands[-1]
        filtered, _ = est.distance_filter.apply(guide.clone(), dist.clone(), W["sigma_i"] / 2, W["sigma_s"] / 2)
        return filtered[0]

    def frame(match, stitch):
        images_p = [im.unsqueeze(0).permute(0, 3, 1, 2).unsqueeze(2) for im in match]
        maps = [distance_of(r, est.selected_cameras[k], images_p, match) for k, r in enumerate(W["refs"])]
        return est.fishey_stitcher.stitch([im.type(torch.uint8) for im in stitch], maps)

    inputs = [([torch.as_tensor(im.astype(np.float32), device=device) for im in f.images_to_match],
               [torch.as_tensor(im.astype(np.float32), device=device) for im in f.images_to_stitch]) for f in frames]
    with torch.no_grad():
        for i in range(max(1, args.warmup)):
            frame(*inputs[i % len(inputs)])
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for i in range(frames_timed):
            frame(*inputs[i % len(inputs)])
        end.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(end) / frames_timed
    return {"value": 1000.0 / ms, "unit": UNIT, "ms_per_frame": ms, "frames": frames_timed,
            "mode": "the reference's torch sweep and selection restated (materialised volumes, grid_sample), "
                    "this library's fp32 ISB filter and stitcher kernels, one frame per call"}


def cpu_baseline(frames_calib, sample_frames: int):
    """The oracle (C restatement of the reference, OpenMP over all cores) on full frames."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import sphere_oracle

    calibration, frames = frames_calib
    W = WORKLOAD
    masks = [np.ones(W["matching"][::-1], np.float32) for _ in range(4)]
    rig = sphere_oracle.OracleRig(calibration, min_dist=W["min_dist"], max_dist=W["max_dist"],
                                  candidate_count=W["candidates"], references_indices=W["refs"], masks=masks,
                                  matching_resolution=W["matching"], rgb_to_stitch_resolution=W["stitch"],
                                  panorama_resolution=W["panorama"], sigma_i=W["sigma_i"], sigma_s=W["sigma_s"])
    inputs = [([im.astype(np.float32) for im in f.images_to_match], [im.astype(np.float32) for im in f.images_to_stitch])
              for f in frames]
    t0 = time.perf_counter()
    for i in range(sample_frames):
        rig.estimate(*inputs[i % len(inputs)])
    dt = time.perf_counter() - t0
    return {"value": sample_frames / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"{sample_frames} full frame(s) of the workload, oracle/sphere_oracle.c (OpenMP, "
                      f"{os.cpu_count()} threads), camera selection and stitcher tables excluded"}


UNEVEN_METRIC = "RGB-D panoramas/s, uneven batch (matching {512,768,1024}^2, {32,64,96} candidates, 3-6 cameras)"


def uneven_jobs(count: int, seed: int = 5000):
    """The uneven workload: ``count`` jobs, each a rig of 3-6 double-sphere cameras on a ring of
    radius 0.1-0.3 m (xi in [-0.3, 0], alpha in [0.5, 0.7]), matching resolution drawn from
    {512^2, 768^2, 1024^2}, candidates from {32, 64, 96}, references cameras 0 and C // 2,
    rgb_to_stitch = matching resolution, panorama 2W x H.  Seeded per job."""
    syn = importlib.import_module(PACKAGE + ".synthetic")
    jobs = []
    for k in range(count):
        rng = np.random.Generator(np.random.PCG64(seed + k))
        width = int(rng.choice([512, 768, 1024]))
        cands = int(rng.choice([32, 64, 96]))
        cams = int(rng.integers(3, 7))
        jobs.append(dict(width=width, candidates=cands, rig=syn.ring_rig(rng, width, cams), refs=[0, cams // 2]))
    return jobs


def uneven_images(jobs, seed: int = 5000):
    """Images of the uneven workload: one seeded scene rendered once per resolution by a 6-camera
    ring, shared by the jobs of that resolution (their own rigs set the work; the image content
    only moves costs and holes around)."""
    syn = importlib.import_module(PACKAGE + ".synthetic")
    pool = {}
    for width in sorted({j["width"] for j in jobs}):
        rng = np.random.Generator(np.random.PCG64(seed + width))
        cams = syn.ring_rig(rng, width, 6)
        scene = syn.random_scene(rng)
        pool[width] = [syn.render_fisheye(scene, c, width, width)[0] for c in cams]
    return [(np.stack(pool[j["width"]][:len(j["rig"])]), np.stack([pool[j["width"]][r] for r in j["refs"]]))
            for j in jobs]


def run_uneven(args, device):
    import torch

    ss = importlib.import_module(PACKAGE)
    syn = importlib.import_module(PACKAGE + ".synthetic")
    uneven = importlib.import_module(PACKAGE + ".uneven")
    autotune = importlib.import_module(PACKAGE + ".autotune")
    jobs = uneven_jobs(args.jobs)
    images = uneven_images(jobs)
    estimators = []
    for j in jobs:
        w = j["width"]
        calibs = ss.parse_json_calib(syn.basalt_calibration(j["rig"]), (w, w), device)
        vp = torch.zeros(3, device=device)
        for r in j["refs"]:
            vp += calibs[r].rt[:3, 3] / len(j["refs"])
        masks = [torch.ones(1, w, w, device=device) for _ in j["rig"]]
        estimators.append(ss.RGBD_Estimator(calibs, 0.55, 100.0, j["candidates"], j["refs"], vp, masks, (w, w),
                                            (w, w), (2 * w, w), 10.0, 25.0, device, cost_storage=args.storage))
    tuner = autotune.Tuner() if not args.no_autotune else None
    batch = uneven.UnevenBatch(estimators, storage=args.storage, cuda_graphs=True, input_dtype=torch.uint8,
                               tuner=tuner)
    for k, (m, st) in enumerate(images):
        batch.match_inputs[k].copy_(torch.as_tensor(m))
        batch.stitch_inputs[k].copy_(torch.as_tensor(st))
    for _ in range(args.warmup):
        batch.run()
    torch.cuda.synchronize()
    with ClockSampler(device.index) as clocks:
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(args.steps):
            batch.run()
        end.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(end) / args.steps
    # end to end: uint8 inputs from pinned host memory, panoramas back, every step.  Uploads (next
    # step) and downloads (previous step) run on their own streams into / out of two device slots,
    # overlapping the batch; a step copies its slot into the batch's inputs and its outputs into
    # a slot on the compute stream.
    pinned = [(torch.as_tensor(m).pin_memory(), torch.as_tensor(st).pin_memory()) for m, st in images]
    outs = batch.run()
    host_out = [[(torch.empty(r.shape, dtype=r.dtype).pin_memory(), torch.empty(d.shape).pin_memory())
                 for r, d in outs] for _ in range(2)]
    in_slots = [[(torch.empty_like(a, device=device), torch.empty_like(b, device=device)) for a, b in pinned]
                for _ in range(2)]
    out_slots = [[(torch.empty_like(r), torch.empty_like(d)) for r, d in outs] for _ in range(2)]
    h2d = sum(a.numel() + b.numel() for a, b in pinned)
    d2h = sum(a.numel() + 4 * b.numel() for a, b in host_out[0])
    compute = torch.cuda.current_stream(device)
    up_stream, down_stream = torch.cuda.Stream(device), torch.cuda.Stream(device)
    uploaded = [torch.cuda.Event() for _ in range(2)]
    consumed = [torch.cuda.Event() for _ in range(2)]
    produced = [torch.cuda.Event() for _ in range(2)]
    downloaded = [torch.cuda.Event() for _ in range(2)]

    def upload(i):
        slot = i % 2
        with torch.cuda.stream(up_stream):
            up_stream.wait_event(consumed[slot])
            for (dm, ds), (m, st) in zip(in_slots[slot], pinned):
                dm.copy_(m, non_blocking=True)
                ds.copy_(st, non_blocking=True)
            uploaded[slot].record(up_stream)

    def e2e(steps):
        for ev in consumed + downloaded:
            ev.record(compute)
        upload(0)
        for i in range(steps):
            if i + 1 < steps:
                upload(i + 1)
            slot = i % 2
            compute.wait_event(uploaded[slot])
            for k, (dm, ds) in enumerate(in_slots[slot]):
                batch.match_inputs[k].copy_(dm, non_blocking=True)
                batch.stitch_inputs[k].copy_(ds, non_blocking=True)
            consumed[slot].record(compute)
            results = batch.run()
            compute.wait_event(downloaded[slot])
            for (r, d), (sr, sd) in zip(results, out_slots[slot]):
                sr.copy_(r, non_blocking=True)
                sd.copy_(d, non_blocking=True)
            produced[slot].record(compute)
            with torch.cuda.stream(down_stream):
                down_stream.wait_event(produced[slot])
                for (sr, sd), (hr, hd) in zip(out_slots[slot], host_out[slot]):
                    hr.copy_(sr, non_blocking=True)
                    hd.copy_(sd, non_blocking=True)
                downloaded[slot].record(down_stream)
        for ev in downloaded:
            compute.wait_event(ev)  # the timed region ends with every output on the host

    e2e(1)
    torch.cuda.synchronize()
    s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s2.record()
    e2e(args.steps)
    e2.record()
    torch.cuda.synchronize()
    e2e_ms = s2.elapsed_time(e2) / args.steps
    mix = {}
    for j in jobs:
        key = f"{j['width']}^2/{j['candidates']}"
        mix[key] = mix.get(key, 0) + 1
    line = {"metric": UNEVEN_METRIC, "value": len(jobs) * 1000.0 / ms, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": f"{args.storage} storage, f32 arithmetic",
            "data": "synthetic: seeded ring rigs per job; one seeded scene per resolution, 8-bit images",
            "config": {"workload": f"{len(jobs)} jobs in one uneven batch, 2 references per rig, panorama 2W x H",
                       "jobs_by_resolution_and_candidates": mix,
                       "instances": batch.instance_count, "launches_per_step": batch.launches(),
                       "mode": "persistent sweep over all instances, CUDA-graph replay", "tuned": batch.tuned},
            "e2e": {"value": len(jobs) * 1000.0 / e2e_ms, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "gpu_launches": batch.launches() * args.steps, "clocks": clocks.summary()}
    print(json.dumps(line))


def use_stream_workload(args):
    """The stream workload: the prototype rig at 1024^2 with 64 candidates, every camera a
    reference, 64 frames per batch (the frames cycle through the rendered pool)."""
    global METRIC, WORKLOAD_NAME
    WORKLOAD.update(candidates=64, refs=[0, 1, 2, 3])
    if args.batch == 8:
        args.batch = 64
    METRIC = "RGB-D panoramas/s @1024\u00b2 match, 64 cand, 4 references, 64-frame batches"
    WORKLOAD_NAME = ("4 double-sphere fisheye cameras (fx=0.28W, xi=-0.2, alpha=0.6) on a 0.2 m square, "
                     "matching 1024x1024, 64 candidates, references 0,1,2,3, rgb_to_stitch 1216x1216, "
                     "panorama 2048x1024, sigma_i 10, sigma_s 25, 64 frames per batch")


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(value: float, world: int, device) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--batch", type=int, default=8, help="frames per step (one batch)")
    ap.add_argument("--storage", choices=["fp16", "unorm16"], default="fp16")
    ap.add_argument("--unique-frames", type=int, default=8, help="distinct rendered frames batches are built from")
    ap.add_argument("--cpu-frames", type=int, default=8, help="frames timed for the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-u8", action="store_true", help="skip the uint8-input end-to-end leg")
    ap.add_argument("--plain-frames", type=int, default=32, help="frames timed on the plain fp32 path (0 = skip)")
    ap.add_argument("--workload", choices=["prototype", "stream", "uneven"], default="prototype",
                    help="prototype: the headline 1024^2 / 32-candidate workload; stream: 64-frame batches, "
                         "64 candidates, every camera a reference; uneven: a mixed batch of jobs")
    ap.add_argument("--jobs", type=int, default=128, help="jobs of the uneven workload")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default launch shapes")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the leg that runs the reference's torch sweep, restated, on the GPU")
    ap.add_argument("--knob", action="append", default=[], metavar="NAME=VALUE",
                    help="fix a launch-shape knob (with --no-autotune; autotune.KNOBS names)")
    ap.add_argument("--overlap-groups", type=int, default=None,
                    help="frame groups whose post-filter and stitch overlap the next group's sweep (default: tuned)")
    args = ap.parse_args()

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local_rank = _env_int("LOCAL_RANK", 0)

    if args.impl == "reference":
        if rank != 0:
            return
        data = render_pool(1, 0, 1, oracle_resize)
        for _ in range(args.warmup):
            cpu_baseline(data, 1)
        base = cpu_baseline(data, max(1, args.steps))
        line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / base["value"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
                "config": {"workload": WORKLOAD_NAME, "mode": "reference algorithm on the host cores"},
                "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    device = torch.device("cuda", local_rank)
    torch.cuda.set_device(device)
    if args.workload == "uneven":
        if world > 1:
            raise SystemExit("the uneven workload runs on one GPU")
        run_uneven(args, device)
        return
    if args.workload == "stream":
        use_stream_workload(args)
    rendered = render_pool(args.unique_frames, rank, world, gpu_resize(device))
    ours = run_ours(args, rank, world, device, rendered)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    plain = run_plain_fp32(args, device, rendered, args.plain_frames) if args.plain_frames > 0 else None
    if plain is not None:
        plain["batched_over_plain"] = ours["value"] / (world * plain["value"])
    written = None
    if args.plain_frames > 0 and not args.no_reference_gpu:
        written = run_torch_sweep_gpu(args, device, rendered, max(2, args.plain_frames // 4))
        written["batched_over_it"] = ours["value"] / (world * written["value"])
    base = None
    if not args.no_cpu_baseline:
        base = cpu_baseline((rendered[0], rendered[1][:1]), args.cpu_frames)
    line = {"metric": METRIC, "value": ours["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ours["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE[args.storage], "data": DATA,
            "config": {"workload": WORKLOAD_NAME, "batch_frames": args.batch,
                       "mode": f"batched, {args.storage} cost volume, fp32 arithmetic, CUDA-graph replay",
                       "tuned": ours["tuned"], "overlap_groups": ours["overlap_groups"],
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "inputs": "images to match: 1216x1216 uint8 renders resized to 1024x1024 float32 (fractional "
                                 "values: staged as 8.8 fixed point); images to stitch: the 1216x1216 renders",
                       "l2": f"each step reads a {args.batch}-frame batch of inputs "
                             f"({args.batch} x {(4 * 1024 * 1024 + len(WORKLOAD['refs']) * 1216 * 1216) * 12 / 1e6:.0f} MB), "
                             "alternating between two batches; both far exceed the 126 MB L2"},
            "e2e": ours["e2e"], "e2e_f32": ours["e2e_f32"], "device_from_decoded_u8": ours["device_from_decoded_u8"],
            "plain_fp32_gpu": plain,
            "torch_sweep_gpu": written,
            "gpu_launches": ours["gpu_launches"], "clocks": ours["clocks"],
            "roofline": ours["roofline"], "cpu_baseline": base}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Batched frame pipeline: many frames of one rig per launch sequence, a 16-bit level-0 cost
volume (coarser levels float32) with fp32 arithmetic, optional CUDA-graph capture.

One batch of F frames runs the per-frame steps of RGBD_Estimator.estimate_RGBD_panorama
(python/depth_estimation.py:205-242) for all F x R (frame, reference) instances at once:

    ssg_stage_images[_u8|_resized] inputs -> footprints + guides of the references      1 launch
                                   (_resized: decoded 8-bit images of any size, resized on the way)
    ssg_sweep_cost_batch           sweep + cost, 16-bit chunked volume                  1
    ssg_isb_filter_batch           L - 1 down and L - 2 up steps, the small levels'     fewer than
                                   steps fused into one launch                          2 L - 3
    ssg_isb_upsample_select_batch  last level + argmin / sub-candidate step             1
    ssg_isb_apply_batch            distance post-filter, fp32, N = 1                    2L - 2
    ssg_reproject_distance_batch_approx  fill + z-buffer                                2
    ssg_inpaint_holes_batch        hole filling: a scan, steps on hole lists, a tail    6
    ssg_merge_panorama_batch_approx panoramas                                           1

so the launch count does not grow with F (about 45 at 1024^2).  Buffers are allocated once for
the largest batch; outputs alias them, as the reference's outputs alias its stitcher buffers.
"""
from __future__ import annotations

import ctypes
import gc
import warnings

import torch

from . import _native as N
from .isb_filter import level_shapes, level_weights

STORAGE = {"fp16": 0, "unorm16": 1}
F32 = 2


class BatchPipeline:
    MAX_GROUPS = 8

    def __init__(self, estimator, max_frames: int, storage: str = "fp16", cuda_graphs: bool = True,
                 tuner=None, overlap_groups: int | None = None, output_slots: int = 1):
        """overlap_groups: the batch's frames are split into this many groups; the distance
        post-filter and the stitch of a group run on a second stream while the next group's sweep
        and cost filter run (1 = one group, no overlap; None = the tuner's pick, or 1 without a
        tuner).  output_slots: the panoramas of consecutive runs go to this many buffers in turn,
        so the outputs of a run stay valid for the next output_slots - 1 runs (1: each run
        overwrites the last, as the reference's outputs alias its stitcher buffers)."""
        if storage not in STORAGE:
            raise ValueError(f"storage must be one of {sorted(STORAGE)}")
        if max_frames < 1:
            raise ValueError("max_frames must be positive")
        if overlap_groups is not None and not 1 <= overlap_groups <= self.MAX_GROUPS:
            raise ValueError(f"overlap_groups must be in [1, {self.MAX_GROUPS}]")
        if not 1 <= output_slots <= 4:
            raise ValueError("output_slots must be in [1, 4]")
        self.overlap_groups = overlap_groups
        e = estimator
        self.e = e
        self.device = e.device
        self.storage = STORAGE[storage]
        self.storage_name = storage
        self.max_frames = max_frames
        self.cuda_graphs = cuda_graphs
        self.cols, self.rows = e.matching_resolution
        self.P = self.cols * self.rows
        self.C = len(e.calibrations)
        self.R = len(e.references_indices)
        self.N = e.candidate_count
        self.chunks = (self.N + 7) // 8
        st = e.fishey_stitcher
        self.st = st
        self.shapes = level_shapes(e.matching_resolution)
        self.L = len(self.shapes)
        F, R, C, P = max_frames, self.R, self.C, self.P
        dev = self.device
        u8 = dict(dtype=torch.uint8, device=dev)
        f32 = dict(dtype=torch.float32, device=dev)
        i16 = dict(dtype=torch.int16, device=dev)
        # two planes (high and low bytes of 8.8 fixed-point codes) of 16-byte bilinear footprints,
        # (rows + 2) x (cols + 2) per camera, and a class per plane (integer / fixed / float)
        self.staged = torch.zeros(F * C * 2 * (self.rows + 2) * (self.cols + 2) * 4, **f32)
        self.plane_flags = torch.zeros(F * C, dtype=torch.int32, device=dev)
        # guides: one 32-bit word per pixel (Y, Cb, Cr, 0)
        self.guides = [torch.empty(F * R * r * c * 4, **u8) for r, c in self.shapes]
        # level 0 (the sweep's output) 16-bit, coarser levels float32
        self.costs = [torch.empty(F * R * self.chunks * r * c * 8, **(i16 if l == 0 else f32))
                      for l, (r, c) in enumerate(self.shapes)]
        # the distance post-filter's guide pyramid; its level 0 is the unfiltered guide itself,
        # which the batched cost filter leaves as it was
        self.df_guides = [self.guides[0]] + [torch.empty(F * R * r * c * 4, **u8) for r, c in self.shapes[1:]]
        self.df_costs = [torch.empty(F * R * r * c, **f32) for r, c in self.shapes[1:]]
        self.distance_raw = torch.empty(F * R * P, **f32)
        self.index = torch.empty(F * R * P, dtype=torch.int32, device=dev)
        self.distance = torch.empty(F, R, self.rows, self.cols, **f32)
        self.reprojected = torch.empty(F * R * P, **f32)
        self.stamps = torch.empty(F * R * P, **u8)
        self.holes = torch.empty(3 * F * R * P + N.HOLE_SCRATCH_HEADER * self.MAX_GROUPS, dtype=torch.int32,
                                 device=dev)
        self.images_u8 = torch.empty(F, R, st.image_rows, st.image_cols, 3, **u8)
        # the panoramas: output_slots buffers used in turn; rgb / pano_distance are the current one
        self._out_slots = [(torch.empty(F, st.pano_rows, st.pano_cols, 3, **u8),
                            torch.empty(F, st.pano_rows, st.pano_cols, **f32)) for _ in range(output_slots)]
        self._next_slot = self._slot = 0
        self.rgb, self.pano_distance = self._out_slots[0]
        self.tables = torch.stack(st.inpainting_weights_list).contiguous()
        self.selected = torch.stack(e._selected).contiguous()
        self._refs = N.ints(e.references_indices)
        self._poses = N.floats([v for r in e.references_indices for v in e._poses_list[r]])
        self._graphs: dict = {}
        self._side = torch.cuda.Stream(dev)  # the post-filter and stitch of overlapped groups
        # decoded 8-bit images of another size than the matching resolution: resized while staging
        # (ssg_stage_images_resized), or, where that kernel declines the shape, resized into this
        # float32 buffer first and staged from it
        self._fused_resize: dict[tuple[int, int, int], bool] = {}
        self._resized: torch.Tensor | None = None
        # launch shapes: picked by the autotuner on first use (``tuner``: an autotune.Tuner, or
        # None for the library's defaults)
        self.tuner = tuner
        self.tuned: dict[str, int] | None = None

    def refresh_rig(self) -> None:
        """Takes the estimator's updated rig (RGBD_Estimator.update_extrinsics): camera selection
        and inpainting tables copied in place, poses re-read, captured graphs dropped (their
        launches hold the old poses as parameters)."""
        e = self.e
        self.selected.copy_(torch.stack(e._selected))
        self.tables.copy_(torch.stack(self.st.inpainting_weights_list))
        self._poses = N.floats([v for r in e.references_indices for v in e._poses_list[r]])
        self._graphs.clear()

    # ------------------------------------------------------------------------------------
    def _estimate(self, match: torch.Tensor, f0: int, frames: int, stream: int) -> None:
        """Staging, sweep, cost filter and selection of frames [f0, f0 + frames)."""
        e = self.e
        R, C, P = self.R, self.C, self.P
        i0, inst = f0 * R, frames * R
        cols, rows = self.cols, self.rows
        plane = (rows + 2) * (cols + 2) * 4  # floats of one plane of footprints (two per camera)
        staged = self.staged.data_ptr() + 4 * f0 * C * 2 * plane
        flags = self.plane_flags.data_ptr() + 4 * f0 * C
        guide0 = self.guides[0].data_ptr() + 4 * i0 * P
        m = match[f0:f0 + frames]
        floats = None
        if match.dtype != torch.uint8:
            # float32 images at the matching resolution: 32-byte entries, class-2 planes sampled from them
            N.call("ssg_stage_images", m.data_ptr(), frames, C, cols, rows, self._refs, R, staged, guide0, flags,
                   stream)
            floats, entry_bytes = m.data_ptr(), 32
        elif m.shape[2:4] == (rows, cols):
            # 8-bit images at the matching resolution: 16-byte entries of bytes
            N.call("ssg_stage_images_u8", m.data_ptr(), frames, C, cols, rows, self._refs, R, staged, guide0, flags,
                   stream)
            entry_bytes = 16
        else:
            # decoded 8-bit images of their own size: resized to the matching resolution (the
            # reference's input preparation, python/utils.py:198-201) while staging
            src_rows, src_cols = m.shape[2], m.shape[3]
            key = (src_cols, src_rows, m.data_ptr() % 4)
            entry_bytes = 32
            if self._fused_resize.get(key, True):
                try:
                    N.call("ssg_stage_images_resized", m.data_ptr(), src_cols, src_rows, frames, C, cols, rows,
                           self._refs, R, staged, guide0, flags, stream)
                    self._fused_resize[key] = True
                except N.SSGError as err:  # declined before any launch: resize first
                    if err.code != N.SSG_ERR_UNSUPPORTED:
                        raise
                    self._fused_resize[key] = False
            if not self._fused_resize[key]:
                if self._resized is None:
                    self._resized = torch.empty(self.max_frames * C * P * 3, dtype=torch.float32, device=self.device)
                resized = self._resized.data_ptr() + 4 * f0 * C * P * 3
                N.call("ssg_resize_linear", m.data_ptr(), N.PIXEL_U8, src_cols, src_rows, 3, resized, N.PIXEL_F32,
                       cols, rows, frames * C, stream)
                N.call("ssg_stage_images", resized, frames, C, cols, rows, self._refs, R, staged, guide0, flags,
                       stream)
                floats = resized
        cell0 = 2 * 8 * self.chunks  # bytes of a level-0 pixel's cells
        N.call("ssg_sweep_cost_batch_entries", cols, rows, frames, C, e._cams, R, self._refs, self._poses, staged,
               entry_bytes, floats, flags, self.selected.data_ptr(), e._candidates, self.N, self.storage,
               self.costs[0].data_ptr() + cell0 * i0 * P, stream)
        var_inv_i = 1 / (2 * e.sigma_i * e.sigma_i)
        L = self.L

        def guide(s):
            r, c = self.shapes[s]
            return self.guides[s].data_ptr() + 4 * i0 * r * c

        def cost(s):
            r, c = self.shapes[s]
            return self.costs[s].data_ptr() + (cell0 if s == 0 else 4 * 8 * self.chunks) * i0 * r * c

        if L >= 2:
            weights = level_weights(L, e.sigma_s)
            N.call("ssg_isb_filter_batch", N.pointers([guide(s) for s in range(L)]),
                   N.pointers([cost(s) for s in range(L)]), L, rows, cols, self.N, inst, self.storage,
                   N.floats([w for w, _ in weights]), N.floats([w for _, w in weights]), var_inv_i, stream)
        # the selection writes the raw distance and, for the post-filter to filter in place, a copy
        dist = self.distance.view(-1)[i0 * P:(i0 + inst) * P]
        raw = self.distance_raw.data_ptr() + 4 * i0 * P
        index = self.index.data_ptr() + 4 * i0 * P
        if L >= 2:
            (rc, cc) = self.shapes[1]
            wu, wd = weights[0]
            N.call("ssg_isb_upsample_select_batch", guide(1), cost(1), rc, cc, guide(0), cost(0), rows, cols, self.N,
                   inst, self.storage, wu, wd, var_inv_i, e._candidates, raw, index, dist.data_ptr(), stream)
        else:
            N.call("ssg_select_distance_batch", cost(0), self.N, P, inst, self.storage, e._candidates, raw, index,
                   stream)
            with torch.cuda.stream(self._stream(stream)):
                dist.copy_(self.distance_raw[i0 * P:(i0 + inst) * P])

    def _finish(self, stitch: torch.Tensor, f0: int, frames: int, group: int, stream: int) -> None:
        """Distance post-filter and stitch of frames [f0, f0 + frames)."""
        e, st = self.e, self.st
        R, P = self.R, self.P
        i0, inst = f0 * R, frames * R
        cols, rows = self.cols, self.rows
        L = self.L
        dist = self.distance.view(-1)[i0 * P:(i0 + inst) * P]
        # distance post-filter on the unfiltered guide (python/depth_estimation.py:200-203)
        if L >= 2:
            df_guides = [self.guides[0].data_ptr() + 4 * i0 * P] + [
                g.data_ptr() + 4 * i0 * r * c for g, (r, c) in zip(self.df_guides[1:], self.shapes[1:])]
            df_costs = [dist.data_ptr()] + [c.data_ptr() + 4 * i0 * r * cc
                                            for c, (r, cc) in zip(self.df_costs, self.shapes[1:])]
            N.call("ssg_isb_apply_batch", N.pointers(df_guides), N.pointers(df_costs), L, rows, cols, 1, inst,
                   float(e.sigma_i) / 2, float(e.sigma_s) / 2, N.ISB_SKIP_FINE_GUIDE, stream)
        # stitch (python/stitcher.py:166-220)
        if stitch is None:
            # the references' own decoded images in the images to match (at the stitch resolution)
            images_u8 = None
        elif stitch.dtype == torch.uint8:
            images_u8 = stitch[f0:f0 + frames]
        else:
            s_img = stitch[f0:f0 + frames]
            images_u8 = self.images_u8[f0:f0 + frames]
            # float -> uint8 truncation (depth_estimation.py:239)
            N.call("ssg_convert_u8", s_img.data_ptr(), images_u8.data_ptr(),
                   frames * R * st.image_rows * st.image_cols * 3, stream)
        reprojected = self.reprojected.data_ptr() + 4 * i0 * P
        N.call("ssg_reproject_distance_batch_approx", dist.data_ptr(), reprojected, cols, rows, inst, R, st._intr,
               st._trans, 1, stream)
        holes = self.holes.data_ptr() + 4 * (3 * i0 * P + N.HOLE_SCRATCH_HEADER * group)
        N.call("ssg_inpaint_holes_batch", reprojected, self.tables.data_ptr(), self.stamps.data_ptr() + i0 * P, holes,
               cols, rows, inst, R, st.max_dist, st.inpainting_iterations, stream)
        if images_u8 is None:
            N.call("ssg_merge_panorama_batch_approx_images", st.blending_sampling.data_ptr(),
                   st.blending_weights.data_ptr(), reprojected, dist.data_ptr(),
                   self._match_images[f0:f0 + frames].data_ptr(), self.C, self._refs, st.image_rows, st.image_cols,
                   st._trans, st._intr, R, cols, rows, st.pano_cols, st.pano_rows, frames,
                   self.pano_distance[f0].data_ptr(), self.rgb[f0].data_ptr(), stream)
        else:
            N.call("ssg_merge_panorama_batch_approx", st.blending_sampling.data_ptr(), st.blending_weights.data_ptr(),
                   reprojected, dist.data_ptr(), images_u8.data_ptr(), st.image_rows, st.image_cols, st._trans,
                   st._intr, R, cols, rows, st.pano_cols, st.pano_rows, frames, self.pano_distance[f0].data_ptr(),
                   self.rgb[f0].data_ptr(), stream)

    def _stream(self, handle: int) -> torch.cuda.Stream:
        if not handle:
            return torch.cuda.default_stream(self.device)
        return torch.cuda.ExternalStream(handle, device=self.device)

    def _groups(self, frames: int, groups: int) -> list[tuple[int, int]]:
        groups = max(1, min(groups, frames))
        base, extra = divmod(frames, groups)
        out, f0 = [], 0
        for g in range(groups):
            n = base + (1 if g < extra else 0)
            out.append((f0, n))
            f0 += n
        return out

    def _group_count(self, frames: int) -> int:
        if self.overlap_groups is not None:
            return self.overlap_groups
        if self.tuned is not None and "overlap_groups" in self.tuned:
            return self.tuned["overlap_groups"]
        return 1

    def _launch(self, match: torch.Tensor, stitch: torch.Tensor, frames: int, stream: int,
                groups: int | None = None) -> None:
        groups = self._group_count(frames) if groups is None else groups
        parts = self._groups(frames, groups)
        if len(parts) == 1:
            self._estimate(match, 0, frames, stream)
            self._finish(stitch, 0, frames, 0, stream)
            return
        main = self._stream(stream)
        side = self._side
        for g, (f0, n) in enumerate(parts):
            self._estimate(match, f0, n, stream)
            ready = torch.cuda.Event()
            ready.record(main)
            side.wait_event(ready)
            self._finish(stitch, f0, n, g, side.cuda_stream)
        done = torch.cuda.Event()
        done.record(side)
        main.wait_event(done)

    def run(self, match: torch.Tensor, stitch: torch.Tensor | None):
        """match: [F, C, rows, cols, 3], stitch: [F, R, image_rows, image_cols, 3], each float32 or
        uint8 (8-bit images: a quarter of the upload, no conversion pass), contiguous on the
        pipeline's device.  An 8-bit `match` may also have its own size [F, C, H, W, 3] (the decoded
        images): it is then resized to the matching resolution, as the reference's input
        preparation resizes (python/utils.py:198-201), while it is staged.  `stitch` may be None when
        `match` holds the decoded 8-bit images at the stitch resolution: the references' images in
        it are stitched in place (the reference's images to stitch are those decoded images, resized
        to their own size).  Returns views of the outputs for F frames."""
        frames = match.shape[0] if match.dim() else 0
        if not 1 <= frames <= self.max_frames:
            raise ValueError(f"batch of {frames} frames outside [1, {self.max_frames}]")
        st = self.st
        match_shape = (frames, self.C, self.rows, self.cols, 3)
        if match.dtype == torch.uint8 and match.dim() == 5 and match.shape[4] == 3 and min(match.shape[2:4]) >= 1:
            match_shape = (frames, self.C, match.shape[2], match.shape[3], 3)
        checks = [("images_to_match", match, match_shape)]
        if stitch is None:
            if match.dtype != torch.uint8 or tuple(match.shape[2:4]) != (st.image_rows, st.image_cols):
                raise ValueError("images_to_stitch may only be omitted when images_to_match are the decoded uint8 "
                                 f"images at the stitch resolution {st.image_cols}x{st.image_rows}")
        else:
            checks.append(("images_to_stitch", stitch, (frames, self.R, st.image_rows, st.image_cols, 3)))
        for name, t, shape in checks:
            N.require(t, name, torch.uint8 if t.dtype == torch.uint8 else torch.float32, shape, self.device)
        self._match_images = match
        self._slot = self._next_slot
        self.rgb, self.pano_distance = self._out_slots[self._slot]
        self._next_slot = (self._slot + 1) % len(self._out_slots)
        self._apply_tuning(match, stitch, frames)
        tma = N.library().ssg_tuning_get(N.TUNE_ISB_TILE_TMA) == 1
        self._run(match, stitch, frames)
        if tma and self._tma_wait_ran_out():
            # a tile never landed: the launch's outputs are incomplete; stage by cp.async from now on
            warnings.warn("a bounded wait for a TMA tile of the ISB upsampling ran out; the batch is run again "
                          "with cp.async staging (SSG_TUNE_ISB_TILE_TMA = 0)", RuntimeWarning, stacklevel=2)
            N.call("ssg_tuning_set", N.TUNE_ISB_TILE_TMA, 0)
            if self.tuned is not None:
                self.tuned["isb_tile_tma"] = 0
            self._graphs.clear()
            self._run(match, stitch, frames)
        return self.rgb[:frames], self.pano_distance[:frames]

    @staticmethod
    def _tma_wait_ran_out() -> bool:
        """Reads (and clears) the library's device status word; synchronises the device."""
        status = ctypes.c_uint32(0)
        N.call("ssg_take_device_status", ctypes.byref(status))
        return bool(status.value & N.STATUS_TMA_TIMEOUT)

    def _run(self, match: torch.Tensor, stitch: torch.Tensor, frames: int) -> None:
        if not self.cuda_graphs:
            self._launch(match, stitch, frames, N.stream_of(match))
        else:
            key = (match.data_ptr(), match.dtype, stitch.data_ptr() if stitch is not None else 0,
                   stitch.dtype if stitch is not None else None, frames, self._group_count(frames))
            graphs = self._graphs.get(key)
            if graphs is None:
                # one eager run (first-use set-up such as shared-memory opt-in happens outside capture)
                self._launch(match, stitch, frames, N.stream_of(match))
                # objects that are already garbage (an earlier graph, say) are freed now: a graph
                # destroyed while this capture runs would invalidate it
                gc.collect()
                # one graph per output slot, all captured now: later runs of these inputs replay,
                # whichever slot their turn falls on
                current = (self.rgb, self.pano_distance)
                graphs = []
                for out in self._out_slots:
                    self.rgb, self.pano_distance = out
                    graph = torch.cuda.CUDAGraph()
                    side = torch.cuda.Stream(self.device)
                    side.wait_stream(torch.cuda.current_stream(self.device))
                    with torch.cuda.stream(side):
                        with torch.cuda.graph(graph, stream=side):
                            self._launch(match, stitch, frames, side.cuda_stream)
                    torch.cuda.current_stream(self.device).wait_stream(side)
                    graphs.append(graph)
                self.rgb, self.pano_distance = current
                if len(self._graphs) >= 8:
                    self._graphs.pop(next(iter(self._graphs)))
                self._graphs[key] = graphs
            graphs[self._slot].replay()

    # in tuning order: a register bound before the staging it pairs with (a staging choice is timed
    # at the bound already picked)
    TUNED_KNOBS = ("sweep_variant", "sweep_tiles", "isb_up_blocks", "up_whole", "isb_select_blocks", "select_whole",
                   "isb_tile_tma", "isb_tail", "post_tail", "hole_blocks_per_sm", "hole_persistent", "hole_tail",
                   "merge_frames")
    GROUP_CHOICES = (1, 2, 4)

    def _apply_tuning(self, match, stitch, frames) -> None:
        """Sets this pipeline's launch shapes (process-wide knobs), tuning them on first use; then
        picks the overlap group count (unless the caller fixed it) by timing whole batches."""
        if self.tuner is None:
            return
        from . import autotune

        if self.tuned is None:
            key = autotune.workload_key("batch", self.cols, self.rows, self.N, self.C, self.R, frames,
                                        self.storage_name, self.st.pano_cols, self.st.pano_rows)
            self.tuned = self.tuner.apply(key)
            stream = N.stream_of(match)
            if self.tuned is None or not set(self.TUNED_KNOBS) <= set(self.tuned):
                self.tuned = self.tuner.tune(key, lambda: self._launch(match, stitch, frames, stream, groups=1),
                                             list(self.TUNED_KNOBS))
            if self.overlap_groups is None and "overlap_groups" not in self.tuned:
                runs = {g: (lambda g=g: self._launch(match, stitch, frames, stream, groups=g))
                        for g in self.GROUP_CHOICES if g <= frames}
                self.tuned["overlap_groups"] = self.tuner.pick(key, "overlap_groups", runs, stream)
        for name, v in self.tuned.items():
            if name in autotune.KNOBS:
                autotune.set_knob(name, v)

    def launches_per_batch(self, frames: int | None = None, float_stitch: bool = True) -> int:
        """Kernels one batch of ``frames`` frames launches (float32 images to stitch add a
        conversion per group)."""
        frames = self.max_frames if frames is None else frames
        L = self.L
        isb = N.isb_filter_launches(self.rows, self.cols, L) + 1 if L >= 2 else 1
        post = N.isb_apply_launches(self.rows, self.cols, L, 1) if L >= 2 else 0
        inpaint = N.hole_filling_launches(self.st.inpainting_iterations)
        per_group = 2 + isb + post + (1 if float_stitch else 0) + 2 + inpaint + 1
        return per_group * len(self._groups(frames, self._group_count(frames)))

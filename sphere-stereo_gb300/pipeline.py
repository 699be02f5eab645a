"""Batched frame pipeline: many frames of one rig per launch sequence, a 16-bit level-0 cost
volume (coarser levels float32) with fp32 arithmetic, optional CUDA-graph capture.

One batch of F frames runs the per-frame steps of RGBD_Estimator.estimate_RGBD_panorama
(python/depth_estimation.py:205-242) for all F x R (frame, reference) instances at once:

    ssg_stage_images[_u8]          inputs -> 8-bit footprints + guides of the references 1 launch
    ssg_sweep_cost_batch           sweep + cost, 16-bit chunked volume                  1
    ssg_isb_downsample_batch       L - 1 levels                                         L - 1
    ssg_isb_upsample_batch         levels L - 2 .. 1                                    L - 2
    ssg_isb_upsample_select_batch  last level + argmin / sub-candidate step             1
    ssg_isb_apply_batch            distance post-filter, fp32, N = 1                    2L - 2
    ssg_reproject_distance_batch   fill + z-buffer                                      2
    ssg_inpaint_holes_batch        hole filling: a scan, then 32 steps on hole lists    33
    ssg_merge_panorama_batch_approx panoramas                                           1

so the launch count does not grow with F (about 70 at 1024^2).  Buffers are allocated once for
the largest batch; outputs alias them, as the reference's outputs alias its stitcher buffers.
"""
from __future__ import annotations

import torch

from . import _native as N
from .isb_filter import level_shapes, level_weights

STORAGE = {"fp16": 0, "unorm16": 1}
F32 = 2


class BatchPipeline:
    def __init__(self, estimator, max_frames: int, storage: str = "fp16", cuda_graphs: bool = True,
                 tuner=None):
        if storage not in STORAGE:
            raise ValueError(f"storage must be one of {sorted(STORAGE)}")
        if max_frames < 1:
            raise ValueError("max_frames must be positive")
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
        # planes of 16-byte bilinear footprints (8-bit RGB), (rows + 2) x (cols + 2) per camera, and
        # a flag per plane for the planes sampled from the float images instead
        self.staged = torch.zeros(F * C * (self.rows + 2) * (self.cols + 2) * 4, **f32)
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
        self.holes = torch.empty(3 * F * R * P + 4, dtype=torch.int32, device=dev)
        self.images_u8 = torch.empty(F, R, st.image_rows, st.image_cols, 3, **u8)
        self.rgb = torch.empty(F, st.pano_rows, st.pano_cols, 3, **u8)
        self.pano_distance = torch.empty(F, st.pano_rows, st.pano_cols, **f32)
        self.tables = torch.stack(st.inpainting_weights_list).contiguous()
        self.selected = torch.stack(e._selected).contiguous()
        self._refs = N.ints(e.references_indices)
        self._poses = N.floats([v for r in e.references_indices for v in e._poses_list[r]])
        self._graphs: dict = {}
        # launch shapes: picked by the autotuner on first use (``tuner``: an autotune.Tuner, or
        # None for the library's defaults)
        self.tuner = tuner
        self.tuned: dict[str, int] | None = None

    # ------------------------------------------------------------------------------------
    def _launch(self, match: torch.Tensor, stitch: torch.Tensor, frames: int, stream: int) -> None:
        e, st = self.e, self.st
        inst = frames * self.R
        cols, rows, P = self.cols, self.rows, self.P
        stage = "ssg_stage_images_u8" if match.dtype == torch.uint8 else "ssg_stage_images"
        N.call(stage, match.data_ptr(), frames, self.C, cols, rows, self._refs, self.R, self.staged.data_ptr(),
               self.guides[0].data_ptr(), self.plane_flags.data_ptr(), stream)
        floats = None if match.dtype == torch.uint8 else match.data_ptr()
        N.call("ssg_sweep_cost_batch", cols, rows, frames, self.C, e._cams, self.R, self._refs, self._poses,
               self.staged.data_ptr(), floats, self.plane_flags.data_ptr(), self.selected.data_ptr(), e._candidates,
               self.N, self.storage, self.costs[0].data_ptr(), stream)
        var_inv_i = 1 / (2 * e.sigma_i * e.sigma_i)
        L = self.L
        if L >= 2:
            weights = level_weights(L, e.sigma_s)
            for s in range(1, L):
                (ri, ci), (ro, co) = self.shapes[s - 1], self.shapes[s]
                N.call("ssg_isb_downsample_batch", self.guides[s - 1].data_ptr(), self.costs[s - 1].data_ptr(), ri, ci,
                       self.guides[s].data_ptr(), self.costs[s].data_ptr(), ro, co, self.N, inst,
                       self.storage if s == 1 else F32, var_inv_i, stream)
            for s in range(L - 2, 0, -1):
                (rc, cc), (rf, cf) = self.shapes[s + 1], self.shapes[s]
                wu, wd = weights[s]
                N.call("ssg_isb_upsample_batch", self.guides[s + 1].data_ptr(), self.costs[s + 1].data_ptr(), rc, cc,
                       self.guides[s].data_ptr(), self.costs[s].data_ptr(), rf, cf, self.N, inst, F32, wu, wd,
                       var_inv_i, stream)
        # the selection writes the raw distance and, for the post-filter to filter in place, a copy
        dist = self.distance.view(-1)[: inst * P]
        if L >= 2:
            (rc, cc) = self.shapes[1]
            wu, wd = weights[0]
            N.call("ssg_isb_upsample_select_batch", self.guides[1].data_ptr(), self.costs[1].data_ptr(), rc, cc,
                   self.guides[0].data_ptr(), self.costs[0].data_ptr(), rows, cols, self.N, inst, self.storage, wu, wd,
                   var_inv_i, e._candidates, self.distance_raw.data_ptr(), self.index.data_ptr(), dist.data_ptr(),
                   stream)
        else:
            N.call("ssg_select_distance_batch", self.costs[0].data_ptr(), self.N, P, inst, self.storage,
                   e._candidates, self.distance_raw.data_ptr(), self.index.data_ptr(), stream)
            dist.copy_(self.distance_raw[: inst * P])
        # distance post-filter on the unfiltered guide (python/depth_estimation.py:200-203)
        if L >= 2:
            N.call("ssg_isb_apply_batch", N.pointers([g.data_ptr() for g in self.df_guides]),
                   N.pointers([dist.data_ptr()] + [c.data_ptr() for c in self.df_costs]), L, rows, cols, 1, inst,
                   float(e.sigma_i) / 2, float(e.sigma_s) / 2, N.ISB_SKIP_FINE_GUIDE, stream)
        # stitch (python/stitcher.py:166-220)
        if stitch.dtype == torch.uint8:
            images_u8 = stitch
        else:
            images_u8 = self.images_u8
            # float -> uint8 truncation (depth_estimation.py:239)
            N.call("ssg_convert_u8", stitch.data_ptr(), images_u8.data_ptr(), frames * self.R * st.image_rows *
                   st.image_cols * 3, stream)
        N.call("ssg_reproject_distance_batch", dist.data_ptr(), self.reprojected.data_ptr(), cols, rows, inst, self.R,
               st._intr, st._trans, 1, stream)
        N.call("ssg_inpaint_holes_batch", self.reprojected.data_ptr(), self.tables.data_ptr(), self.stamps.data_ptr(),
               self.holes.data_ptr(), cols, rows, inst, self.R, st.max_dist, st.inpainting_iterations, stream)
        N.call("ssg_merge_panorama_batch_approx", st.blending_sampling.data_ptr(), st.blending_weights.data_ptr(),
               self.reprojected.data_ptr(), dist.data_ptr(), images_u8.data_ptr(), st.image_rows, st.image_cols,
               st._trans, st._intr, self.R, cols, rows, st.pano_cols, st.pano_rows, frames,
               self.pano_distance.data_ptr(), self.rgb.data_ptr(), stream)

    def run(self, match: torch.Tensor, stitch: torch.Tensor):
        """match: [F, C, rows, cols, 3], stitch: [F, R, image_rows, image_cols, 3], each float32 or
        uint8 (8-bit images: a quarter of the upload, no conversion pass), contiguous on the
        pipeline's device.  Returns views of the outputs for F frames."""
        frames = match.shape[0]
        if not 1 <= frames <= self.max_frames:
            raise ValueError(f"batch of {frames} frames outside [1, {self.max_frames}]")
        st = self.st
        for name, t, shape in (("images_to_match", match, (frames, self.C, self.rows, self.cols, 3)),
                               ("images_to_stitch", stitch, (frames, self.R, st.image_rows, st.image_cols, 3))):
            N.require(t, name, torch.uint8 if t.dtype == torch.uint8 else torch.float32, shape, self.device)
        self._apply_tuning(match, stitch, frames)
        if not self.cuda_graphs:
            self._launch(match, stitch, frames, N.stream_of(match))
        else:
            key = (match.data_ptr(), match.dtype, stitch.data_ptr(), stitch.dtype, frames)
            graph = self._graphs.get(key)
            if graph is None:
                # one eager run (first-use set-up such as shared-memory opt-in happens outside capture)
                self._launch(match, stitch, frames, N.stream_of(match))
                graph = torch.cuda.CUDAGraph()
                side = torch.cuda.Stream(self.device)
                side.wait_stream(torch.cuda.current_stream(self.device))
                with torch.cuda.stream(side):
                    with torch.cuda.graph(graph, stream=side):
                        self._launch(match, stitch, frames, side.cuda_stream)
                torch.cuda.current_stream(self.device).wait_stream(side)
                if len(self._graphs) >= 8:
                    self._graphs.pop(next(iter(self._graphs)))
                self._graphs[key] = graph
            graph.replay()
        return self.rgb[:frames], self.pano_distance[:frames]

    TUNED_KNOBS = ("sweep_variant", "isb_up_blocks", "hole_blocks_per_sm", "merge_frames")

    def _apply_tuning(self, match, stitch, frames) -> None:
        """Sets this pipeline's launch shapes (process-wide knobs), tuning them on first use."""
        if self.tuner is None:
            return
        from . import autotune

        if self.tuned is None:
            key = autotune.workload_key("batch", self.cols, self.rows, self.N, self.C, self.R, frames,
                                        self.storage_name, self.st.pano_cols, self.st.pano_rows)
            self.tuned = self.tuner.apply(key)
            if self.tuned is None:
                stream = N.stream_of(match)
                self.tuned = self.tuner.tune(key, lambda: self._launch(match, stitch, frames, stream),
                                             list(self.TUNED_KNOBS))
        for name, v in self.tuned.items():
            autotune.set_knob(name, v)

    def launches_per_batch(self) -> int:
        L = self.L
        isb = (L - 1) + (L - 2) + 1 if L >= 2 else 1
        post = 2 * (L - 1) if L >= 2 else 0
        it = self.st.inpainting_iterations
        inpaint = 0 if it == 0 else 1 + it
        return 2 + isb + post + 2 + inpaint + 1

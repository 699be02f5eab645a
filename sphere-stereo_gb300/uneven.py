"""UnevenBatch: many RGB-D panorama jobs of different rigs, matching resolutions and candidate
counts in one fixed launch sequence (no counterpart in the reference, which estimates one rig's
frame per call of estimate_RGBD_panorama, python/depth_estimation.py:205-242).

Each job is one frame of one rig, described by an RGBD_Estimator built for that rig (camera
selection, candidates and stitcher tables come from it).  Per batch:

    ssg_stage_images[_u8]    one launch per job (inputs -> 8-bit footprint planes + guides)
    ssg_uneven_run           one persistent sweep launch over every instance, one launch per
                             cost-filter and post-filter step, the fused selection, then fill,
                             reprojection, hole lists and merge over every job

The inputs are written into this object's buffers (``match_inputs`` / ``stitch_inputs``, or
through ``run``), so the whole sequence is captured once in a CUDA graph and replayed.
"""
from __future__ import annotations

import ctypes
import gc

import torch

from . import _native as N
from .isb_filter import level_shapes

STORAGE = {"fp16": 0, "unorm16": 1}


class UnevenBatch:
    def __init__(self, estimators, storage: str = "fp16", cuda_graphs: bool = True, input_dtype=torch.float32,
                 tuner=None):
        """Args:
            estimators: one RGBD_Estimator per job (rigs, resolutions and candidate counts may all
                differ); the jobs run together on the estimators' common device
            storage: "fp16" or "unorm16" level-0 cost storage (fp32 arithmetic)
            cuda_graphs: replay the batch from a captured CUDA graph
            input_dtype: torch.float32 (images in [0, 255], as estimate_RGBD_panorama takes them)
                or torch.uint8 (the 8-bit images they are made from)
            tuner: an autotune.Tuner that picks the sweep's block shape and work-item span on
                first use (None: the library's defaults)
        """
        if not estimators:
            raise ValueError("at least one job is required")
        if storage not in STORAGE:
            raise ValueError(f"storage must be one of {sorted(STORAGE)}")
        if input_dtype not in (torch.float32, torch.uint8):
            raise ValueError("input_dtype must be torch.float32 or torch.uint8")
        dev = estimators[0].device
        if any(e.device != dev for e in estimators):
            raise ValueError("all jobs must be on one device")
        self.device = dev
        self.estimators = list(estimators)
        self.storage = STORAGE[storage]
        self.cuda_graphs = cuda_graphs
        self.input_dtype = input_dtype
        u8 = dict(dtype=torch.uint8, device=dev)
        f32 = dict(dtype=torch.float32, device=dev)
        self.match_inputs, self.stitch_inputs = [], []
        self._jobs = []  # per job: buffers and host arrays kept alive for the plan
        instances, jobs = [], []
        self._keep = []
        for e in self.estimators:
            cols, rows = e.matching_resolution
            C, R, n = len(e.calibrations), len(e.references_indices), e.candidate_count
            st = e.fishey_stitcher
            chunks = (n + 7) // 8
            shapes = level_shapes(e.matching_resolution)
            if len(shapes) < 2:
                raise ValueError(f"a {cols}x{rows} job has fewer than two filter levels")
            j = {
                "match": torch.zeros(C, rows, cols, 3, dtype=input_dtype, device=dev),
                "stitch": torch.zeros(R, st.image_rows, st.image_cols, 3, dtype=input_dtype, device=dev),
                "staged": torch.zeros(C * 2 * (rows + 2) * (cols + 2) * 4, **f32),  # high and low planes
                "flags": torch.zeros(C, dtype=torch.int32, device=dev),
                "guide0": torch.empty(R * rows * cols * 4, **u8),  # 32-bit guide words
                "distance": torch.empty(R, rows, cols, **f32),
                "rgb": torch.empty(st.pano_rows, st.pano_cols, 3, **u8),
                "pano_distance": torch.empty(st.pano_rows, st.pano_cols, **f32),
                "images_u8": st.images_to_stitch if input_dtype != torch.uint8 else None,
                "refs": N.ints(e.references_indices),
            }
            j["tables"] = torch.stack(st.inpainting_weights_list).contiguous()
            j["instances"] = []
            for slot, r in enumerate(e.references_indices):
                P = rows * cols
                guides = [j["guide0"][slot * P * 4:(slot + 1) * P * 4]] + \
                    [torch.empty(rr * cc * 4, **u8) for rr, cc in shapes[1:]]
                costs = [torch.empty(chunks * P * 8, dtype=torch.int16, device=dev)] + \
                    [torch.empty(chunks * rr * cc * 8, **f32) for rr, cc in shapes[1:]]
                df_guides = [guides[0]] + [torch.empty(rr * cc * 4, **u8) for rr, cc in shapes[1:]]
                df_costs = [torch.empty(rr * cc, **f32) for rr, cc in shapes[1:]]
                raw = torch.empty(rows, cols, **f32)
                index = torch.empty(rows, cols, dtype=torch.int32, device=dev)
                arrays = {
                    "guides": N.pointers([g.data_ptr() for g in guides]),
                    "costs": N.pointers([c.data_ptr() for c in costs]),
                    "df_guides": N.pointers([g.data_ptr() for g in df_guides]),
                    "df_costs": N.pointers([c.data_ptr() for c in df_costs]),
                    "poses": e._poses[r],
                    "candidates": e._candidates,
                    "cams": e._cams,
                }
                inst = N.ssg_uneven_instance(
                    cols=cols, rows=rows, camera_count=C, reference_camera=r, candidate_count=n,
                    cameras=ctypes.cast(arrays["cams"], ctypes.c_void_p),
                    relative_poses=ctypes.cast(arrays["poses"], ctypes.c_void_p),
                    candidates=ctypes.cast(arrays["candidates"], ctypes.c_void_p),
                    sigma_i=float(e.sigma_i), sigma_s=float(e.sigma_s),
                    d_staged=j["staged"].data_ptr(),
                    d_images=None if input_dtype == torch.uint8 else j["match"].data_ptr(),
                    d_plane_flags=j["flags"].data_ptr(), d_selected=e._selected[slot].data_ptr(),
                    d_guides=ctypes.cast(arrays["guides"], ctypes.c_void_p),
                    d_costs=ctypes.cast(arrays["costs"], ctypes.c_void_p),
                    d_df_guides=ctypes.cast(arrays["df_guides"], ctypes.c_void_p),
                    d_df_costs=ctypes.cast(arrays["df_costs"], ctypes.c_void_p),
                    d_distance_raw=raw.data_ptr(), d_distance=j["distance"][slot].data_ptr(),
                    d_index=index.data_ptr())
                instances.append(inst)
                j["instances"].append({"guides": guides, "costs": costs, "df_guides": df_guides,
                                       "df_costs": df_costs, "raw": raw, "index": index, "arrays": arrays})
            images = j["stitch"] if input_dtype == torch.uint8 else j["images_u8"]
            jobs.append(N.ssg_uneven_job(
                cols=cols, rows=rows, references=R, pano_cols=st.pano_cols, pano_rows=st.pano_rows,
                image_cols=st.image_cols, image_rows=st.image_rows,
                intrinsics=ctypes.cast(st._intr, ctypes.c_void_p), translations=ctypes.cast(st._trans, ctypes.c_void_p),
                d_distance=j["distance"].data_ptr(), d_tables=j["tables"].data_ptr(),
                d_lut=st.blending_sampling.data_ptr(), d_weights=st.blending_weights.data_ptr(),
                d_images=images.data_ptr(), d_pano_distance=j["pano_distance"].data_ptr(), d_rgb=j["rgb"].data_ptr()))
            self._jobs.append(j)
            self.match_inputs.append(j["match"])
            self.stitch_inputs.append(j["stitch"])
        self._instances = (N.ssg_uneven_instance * len(instances))(*instances)
        self._job_specs = (N.ssg_uneven_job * len(jobs))(*jobs)
        plan_bytes, scratch_bytes = ctypes.c_size_t(0), ctypes.c_size_t(0)
        handle = ctypes.c_void_p()
        st0 = self.estimators[0].fishey_stitcher
        N.call("ssg_uneven_create", self._instances, len(instances), self._job_specs, len(jobs), self.storage,
               float(st0.max_dist), int(st0.inpainting_iterations), ctypes.byref(plan_bytes),
               ctypes.byref(scratch_bytes), ctypes.byref(handle))
        self._handle = handle
        # 256-byte aligned device buffers (torch's allocations are)
        self._plan = torch.empty(plan_bytes.value, **u8)
        self._scratch = torch.empty(scratch_bytes.value, **u8)
        stream = torch.cuda.current_stream(dev).cuda_stream
        N.call("ssg_uneven_upload", self._handle, self._plan.data_ptr(), self._scratch.data_ptr(), stream)
        self.instance_count = len(instances)
        self._graph = None
        self.tuner = tuner
        self.tuned: dict[str, int] | None = None

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                N.library().ssg_uneven_destroy(h)
            except Exception:
                pass
            self._handle = None

    # ------------------------------------------------------------------------------------
    def _launch(self, stream: int) -> None:
        for e, j in zip(self.estimators, self._jobs):
            cols, rows = e.matching_resolution
            stage = "ssg_stage_images_u8" if self.input_dtype == torch.uint8 else "ssg_stage_images"
            N.call(stage, j["match"].data_ptr(), 1, len(e.calibrations), cols, rows, j["refs"],
                   len(e.references_indices), j["staged"].data_ptr(), j["guide0"].data_ptr(), j["flags"].data_ptr(),
                   stream)
            if j["images_u8"] is not None:
                # float -> uint8 truncation (depth_estimation.py:239)
                N.call("ssg_convert_u8", j["stitch"].data_ptr(), j["images_u8"].data_ptr(), j["stitch"].numel(),
                       stream)
        N.call("ssg_uneven_run", self._handle, stream)

    def _apply_tuning(self, stream: int) -> None:
        if self.tuner is None:
            return
        from . import autotune

        if self.tuned is None:
            shapes = [(e.matching_resolution, e.candidate_count, len(e.calibrations), len(e.references_indices))
                      for e in self.estimators]
            key = autotune.workload_key("uneven", self.storage, self.input_dtype, shapes)
            self.tuned = self.tuner.apply(key)
            if self.tuned is None:
                self.tuned = self.tuner.tune(key, lambda: self._launch(stream),
                                             ["sweep_variant", "uneven_span", "isb_up_blocks", "isb_select_blocks"],
                                             entry="ssg_uneven_run")
        for name, v in self.tuned.items():
            if name in autotune.KNOBS:
                autotune.set_knob(name, v)

    def launches(self) -> int:
        """Kernels one batch launches."""
        per_job = 1 + (0 if self.input_dtype == torch.uint8 else 1)
        return per_job * len(self._jobs) + N.library().ssg_uneven_launches(self._handle)

    def run(self, images_to_match=None, images_to_stitch=None):
        """Runs every job.  images_to_match[j]: [cameras, rows, cols, 3], images_to_stitch[j]:
        [references, image_rows, image_cols, 3] of ``input_dtype`` (copied into ``match_inputs`` /
        ``stitch_inputs``; pass None when those buffers were filled directly).  Returns one
        (rgb [pano_rows, pano_cols, 3] uint8, distance [pano_rows, pano_cols] float32) per job,
        views of this object's buffers."""
        for name, given, mine in (("images_to_match", images_to_match, self.match_inputs),
                                  ("images_to_stitch", images_to_stitch, self.stitch_inputs)):
            if given is None:
                continue
            if len(given) != len(mine):
                raise ValueError(f"{name}: expected {len(mine)} jobs")
            for t, m in zip(given, mine):
                N.require(t, name, self.input_dtype, tuple(m.shape), self.device)
                m.copy_(t, non_blocking=True)
        stream = torch.cuda.current_stream(self.device)
        self._apply_tuning(stream.cuda_stream)
        if not self.cuda_graphs:
            self._launch(stream.cuda_stream)
        else:
            if self._graph is None:
                self._launch(stream.cuda_stream)  # first use outside the capture
                # objects that are already garbage (an earlier graph, say) are freed now: a graph
                # destroyed while this capture runs would invalidate it
                gc.collect()
                graph = torch.cuda.CUDAGraph()
                side = torch.cuda.Stream(self.device)
                side.wait_stream(stream)
                with torch.cuda.stream(side):
                    with torch.cuda.graph(graph, stream=side):
                        self._launch(side.cuda_stream)
                stream.wait_stream(side)
                self._graph = graph
            self._graph.replay()
        return [(j["rgb"], j["pano_distance"]) for j in self._jobs]

    @property
    def distance_maps(self):
        """Per job, the filtered distance maps of its references, [references, rows, cols]."""
        return [j["distance"] for j in self._jobs]

    @property
    def index_maps(self):
        """Per job, the selected candidate index of each reference, [references, rows, cols]."""
        return [torch.stack([i["index"] for i in j["instances"]]) for j in self._jobs]

    @property
    def raw_distance_maps(self):
        """Per job, the selection's distance before the post-filter, [references, rows, cols]."""
        return [torch.stack([i["raw"] for i in j["instances"]]) for j in self._jobs]

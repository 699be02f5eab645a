"""RGBD_Estimator: RGB-D panoramas from multiview fisheye images by sphere sweeping
(python/depth_estimation.py:38-243), same constructor, methods and return conventions.

Per reference camera and frame the reference runs ~20 torch operations per camera over
[N, H, W, 3] volumes, the ISB filter, ~15 torch reductions and a second filter.  Here that is:

    rgb_to_guide            guide = rgb2yCbCr(image).uint8                      (1 launch)
    ssg_sweep_cost          fused sweep + L1 cost, [N, H, W] float32            (1 launch)
    ssg_isb_downsample      L - 1 levels                                         (L - 1 launches)
    ssg_isb_upsample        levels L - 2 .. 1                                    (L - 2 launches)
    ssg_isb_upsample_select last level fused with argmin / sub-candidate step    (1 launch)
    ssg_isb_apply           distance post-filter (N = 1, sigma / 2)             (2L - 2 launches)

followed by the stitcher (reproject + inpaint per reference, one merge).  Every launch goes on
the caller's current CUDA stream; nothing synchronises the host, so a whole frame can be
captured in a CUDA graph.

Inputs are validated before any launch (shapes, dtypes, devices, contiguity, candidate and
camera limits); the reference performs no such checks.
"""
from __future__ import annotations

import torch

from . import _native as N
from .isb_filter import ISB_Filter, level_shapes, level_weights
from .stitcher import Stitcher
from .utils import _cpu32, camera_struct, relative_poses, rgb_to_guide


def distance_candidates(min_dist, max_dist, candidate_count) -> torch.Tensor:
    """1 / linspace(1 / min_dist, 1 / max_dist, N) in float32 on the CPU
    (python/depth_estimation.py:145-146)."""
    return 1 / torch.linspace(1 / min_dist, 1 / max_dist, candidate_count)


class RGBD_Estimator:
    def __init__(self, calibrations, min_dist, max_dist, candidate_count, references_indices, reprojection_viewpoint,
                 masks, matching_resolution, rgb_to_stitch_resolution, panorama_resolution, sigma_i, sigma_s, device,
                 *, cost_storage="fp32", max_batch=1, cuda_graphs=True, tuner=None, output_slots=1):
        """Prepare RGB-D estimation: camera selection for adaptive matching, filters, stitcher.

        Args:
            calibrations: [cameras] double-sphere calibrations
            min_dist, max_dist: distance range of the sphere sweep
            candidate_count: number of distance candidates between min_dist and max_dist
            references_indices: [references] cameras where distance is estimated before stitching
            reprojection_viewpoint: [3] viewpoint of the output panorama
            masks: [cameras][1, matching_rows, matching_cols] valid areas (1 = reliable)
            matching_resolution: (cols, rows) used for matching
            rgb_to_stitch_resolution: (cols, rows) of the colour images sampled while stitching
            panorama_resolution: (cols, rows) of the output panoramas
            sigma_i: edge preservation of the cost filter (lower preserves edges more)
            sigma_s: smoothing of the cost filter (higher favours coarser scales)
            device: CUDA device
            cost_storage (keyword only, not in the reference): "fp32" runs the reference's
                arithmetic bit for bit against the oracle; "fp16" / "unorm16" store the cost
                volume with 16 bits per candidate (fp32 arithmetic) and run frames in batches
            max_batch (keyword only): largest batch of ``estimate_RGBD_panoramas``
            output_slots (keyword only): ``estimate_RGBD_panoramas`` writes its panoramas to this
                many buffers in turn, so a batch's outputs stay valid while the next
                output_slots - 1 batches run (for a caller that downloads one batch while the
                next computes); 1 = every call overwrites the last, as in the reference
            cuda_graphs (keyword only): replay each batch from a captured CUDA graph
            tuner (keyword only): an autotune.Tuner that picks the batched kernels' launch
                shapes on first use (None: the library's defaults)
        """
        device = torch.device(device)
        if device.type != "cuda":
            raise ValueError(f"RGBD_Estimator runs on a CUDA device, got {device}; there is no CPU path")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        N.library()
        if not 1 <= len(calibrations) <= N.MAX_CAMERAS:
            raise ValueError(f"between 1 and {N.MAX_CAMERAS} cameras are supported")
        if not 1 <= candidate_count <= N.MAX_CANDIDATES:
            raise ValueError(f"candidate_count must be in [1, {N.MAX_CANDIDATES}]")
        if len(masks) != len(calibrations):
            raise ValueError("one mask per camera is required")
        for r in references_indices:
            if not 0 <= r < len(calibrations):
                raise ValueError(f"reference index {r} out of range")
        self.calibrations = calibrations
        self.min_dist = min_dist
        self.max_dist = max_dist
        self.candidate_count = candidate_count
        self.references_indices = list(references_indices)
        self.reprojection_viewpoint = reprojection_viewpoint
        self.matching_resolution = tuple(matching_resolution)
        self.device = device
        self.sigma_i = sigma_i
        self.sigma_s = sigma_s

        if cost_storage not in ("fp32", "fp16", "unorm16"):
            raise ValueError("cost_storage must be 'fp32', 'fp16' or 'unorm16'")
        # the fp32 path's filters (pyramids of candidate_count float32 planes) are allocated on
        # first use: the 16-bit paths have their own buffers
        self._cost_filter = None
        self._distance_filter = None
        calibrations_for_stitch = [calibrations[r] for r in self.references_indices]
        masks_for_stitching = [masks[r] for r in self.references_indices]
        self.fishey_stitcher = Stitcher(calibrations_for_stitch, reprojection_viewpoint, masks_for_stitching, min_dist,
                                        max_dist, matching_resolution, rgb_to_stitch_resolution, panorama_resolution,
                                        device)

        self.distance_candidates_host = distance_candidates(min_dist, max_dist, candidate_count)
        self._candidates = N.floats(self.distance_candidates_host.tolist())
        self._cams = N.cameras_array([camera_struct(c) for c in calibrations])
        self._poses_list = {r: relative_poses(calibrations, r) for r in self.references_indices}
        self._poses = {r: N.floats(v) for r, v in self._poses_list.items()}
        cols, rows = self.matching_resolution
        self._shapes = level_shapes(self.matching_resolution)
        self._guide = torch.empty([rows, cols, 3], dtype=torch.uint8, device=device)
        # per reference: the distance map before the post-filter (depth_estimation.py:196-198)
        self.distance_raw_maps = torch.empty([len(self.references_indices), rows, cols], device=device)
        # per reference: the selected candidate index (torch.min's index, depth_estimation.py:180)
        self.index_maps = torch.empty([len(self.references_indices), rows, cols], dtype=torch.int32, device=device)
        self._masks = masks  # kept for re-selection after a rig update
        self.select_camera(masks)
        self.cost_storage = cost_storage
        self.max_batch = int(max_batch)
        self.cuda_graphs = bool(cuda_graphs)
        self.tuner = tuner
        self.output_slots = int(output_slots)
        self._pipeline = None

    @property
    def cost_filter(self) -> ISB_Filter:
        """The fp32 path's cost filter (python/depth_estimation.py:67)."""
        if self._cost_filter is None:
            self._cost_filter = ISB_Filter(self.candidate_count, self.matching_resolution, self.device)
        return self._cost_filter

    @property
    def distance_filter(self) -> ISB_Filter:
        """The fp32 path's distance post-filter (python/depth_estimation.py:68)."""
        if self._distance_filter is None:
            self._distance_filter = ISB_Filter(1, self.matching_resolution, self.device)
        return self._distance_filter

    def set_rig_tables(self, selected_cameras=None, relative_poses=None):
        """Replace the per-rig tables computed at construction (no counterpart in the reference,
        which recomputes poses with torch on every call).

        Args:
            selected_cameras: per reference, [1, rows, cols] or [rows, cols] integer camera
                indices (-1 = none), e.g. another implementation's ``selected_cameras``
            relative_poses: per reference, camera_count x 12 floats: rows 0..2 of
                inverse(camera.rt) @ reference.rt (python/depth_estimation.py:156)
        The tables are host-computed with float32 linear algebra whose last bit depends on the
        platform's BLAS; the selection compares displacements and can flip on exact ties, so
        parity checks against another platform's outputs pass that platform's tables in here.
        """
        cols, rows = self.matching_resolution
        if selected_cameras is not None:
            if len(selected_cameras) != len(self.references_indices):
                raise ValueError("one selection map per reference is required")
            sel8 = []
            for s_ in selected_cameras:
                t = torch.as_tensor(s_).reshape(rows, cols).to(self.device)
                if t.min() < -1 or t.max() >= len(self.calibrations):
                    raise ValueError("camera indices out of range")
                sel8.append(t.to(torch.int8).contiguous())
            self._selected = sel8
            self.selected_cameras = [t.long().unsqueeze(0) for t in sel8]
        if relative_poses is not None:
            if len(relative_poses) != len(self.references_indices):
                raise ValueError("one pose table per reference is required")
            for r, v in zip(self.references_indices, relative_poses):
                v = [float(x) for x in torch.as_tensor(v).reshape(-1).tolist()]
                if len(v) != 12 * len(self.calibrations):
                    raise ValueError("each pose table needs camera_count x 12 floats")
                self._poses_list[r] = v
                self._poses[r] = N.floats(v)
        self._pipeline = None

    def pipeline(self):
        """The batched 16-bit pipeline (built on first use)."""
        if self._pipeline is None:
            from .pipeline import BatchPipeline

            storage = "fp16" if self.cost_storage == "fp32" else self.cost_storage
            self._pipeline = BatchPipeline(self, self.max_batch, storage, self.cuda_graphs, self.tuner,
                                           output_slots=self.output_slots)
        return self._pipeline

    # --------------------------------------------------------------------------------------
    def update_extrinsics(self, rts=None, reprojection_viewpoint=None) -> None:
        """Calibration refinement without rebuilding the estimator (no counterpart in the
        reference, which fixes the rig in its constructor): new camera -> rig poses ``rts``
        (one [4, 4] per camera; None keeps them) and/or a new ``reprojection_viewpoint``.

        Recomputes what depends on them, on the GPU and in place: the relative poses of the
        sweep, the camera selection (python/depth_estimation.py:83-135) and the stitcher's
        translations, inpainting tables, blending LUT and weights (python/stitcher.py:126-164).
        Intrinsics, resolutions, masks, buffers and tuned launch shapes stay; the batched
        pipeline's captured graphs are dropped and recaptured on the next batch.  Results equal
        those of an estimator constructed with the new poses.  An UnevenBatch built from this
        estimator holds the old poses in its descriptors and must be rebuilt."""
        if rts is not None:
            if len(rts) != len(self.calibrations):
                raise ValueError(f"expected {len(self.calibrations)} poses, got {len(rts)}")
            new = []
            for c, rt in zip(self.calibrations, rts):
                t = torch.as_tensor(rt, dtype=torch.float32)
                if tuple(t.shape) != (4, 4) or not bool(torch.isfinite(t).all()):
                    raise ValueError("each pose must be a finite [4, 4] matrix")
                new.append(t.to(c.rt.device) if isinstance(c.rt, torch.Tensor) else t)
            for c, t in zip(self.calibrations, new):
                c.rt = t
            self._poses_list = {r: relative_poses(self.calibrations, r) for r in self.references_indices}
            self._poses = {r: N.floats(v) for r, v in self._poses_list.items()}
            self.select_camera(self._masks)
        if reprojection_viewpoint is not None:
            self.reprojection_viewpoint = reprojection_viewpoint
        self.fishey_stitcher.update_extrinsics([self.calibrations[r] for r in self.references_indices],
                                               self.reprojection_viewpoint)
        if self._pipeline is not None:
            self._pipeline.refresh_rig()

    def select_camera(self, masks):
        """Per reference pixel, the camera with the largest near-far displacement
        (python/depth_estimation.py:83-135).  Fills ``selected_cameras`` ([1, rows, cols] int64,
        -1 where no camera qualifies) like the reference."""
        cols, rows = self.matching_resolution
        mask_stack = torch.stack([torch.as_tensor(m, dtype=torch.float32).reshape(rows, cols) for m in masks])
        mask_stack = mask_stack.to(self.device).contiguous()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        self._selected = []
        self.selected_cameras = []
        for r in self.references_indices:
            sel = torch.empty([rows, cols], dtype=torch.int8, device=self.device)
            N.call("ssg_select_camera", cols, rows, len(self.calibrations), self._cams, r, self._poses[r],
                   mask_stack.data_ptr(), float(self.min_dist), float(self.max_dist), sel.data_ptr(), stream)
            self._selected.append(sel)
            self.selected_cameras.append(sel.long().unsqueeze(0))

    # --------------------------------------------------------------------------------------
    def _validate_images(self, images, shape, name):
        for i, im in enumerate(images):
            N.require(im, f"{name}[{i}]", torch.float32, shape, self.device)

    def _distance(self, slot: int, reference: int, guide: torch.Tensor, images, out: torch.Tensor) -> torch.Tensor:
        """Filtered distance map of one reference camera into ``out`` ([rows, cols] float32)
        (python/depth_estimation.py:137-203)."""
        cols, rows = self.matching_resolution
        n = self.candidate_count
        stream = N.stream_of(guide)
        cf = self.cost_filter
        cost = cf.costs[0]
        guides = cf.guides
        costs = [cost] + cf.costs[1:]
        N.call("ssg_sweep_cost", cols, rows, len(self.calibrations), self._cams, reference, self._poses[reference],
               N.pointers([im.data_ptr() for im in images]), self._selected[slot].data_ptr(), self._candidates, n,
               cost.data_ptr(), stream)
        # cost filter on a copy of the guide (python/depth_estimation.py:177)
        guides[0].copy_(guide)
        L = len(self._shapes)
        var_inv_i = 1 / (2 * self.sigma_i * self.sigma_i)
        raw = self.distance_raw_maps[slot]
        if L >= 2:
            weights = level_weights(L, self.sigma_s)
            for s in range(1, L):
                (ri, ci), (ro, co) = self._shapes[s - 1], self._shapes[s]
                N.call("ssg_isb_downsample", guides[s - 1].data_ptr(), costs[s - 1].data_ptr(), ri, ci,
                       guides[s].data_ptr(), costs[s].data_ptr(), ro, co, n, var_inv_i, stream)
            for s in range(L - 2, 0, -1):
                (rc, cc), (rf, cfn) = self._shapes[s + 1], self._shapes[s]
                wu, wd = weights[s]
                N.call("ssg_isb_upsample", guides[s + 1].data_ptr(), costs[s + 1].data_ptr(), rc, cc,
                       guides[s].data_ptr(), costs[s].data_ptr(), rf, cfn, n, wu, wd, var_inv_i, stream)
            (rc, cc) = self._shapes[1]
            wu, wd = weights[0]
            N.call("ssg_isb_upsample_select", guides[1].data_ptr(), costs[1].data_ptr(), rc, cc,
                   guides[0].data_ptr(), cost.data_ptr(), rows, cols, n, wu, wd, var_inv_i, self._candidates,
                   raw.data_ptr(), self.index_maps[slot].data_ptr(), stream)
        else:
            N.call("ssg_select_distance", cost.data_ptr(), n, rows * cols, self._candidates, raw.data_ptr(),
                   self.index_maps[slot].data_ptr(), stream)
        # distance post-filter with higher edge preservation (python/depth_estimation.py:200-203)
        df = self.distance_filter
        df.guides[0].copy_(guide)
        out3 = out.view(1, rows, cols)
        out3.copy_(raw.view(1, rows, cols))
        df.apply(df.guides[0], out3, self.sigma_i / 2, self.sigma_s / 2)
        return out

    def estimate_fisheye_distance(self, reference_image, guide, reference_calibration, selected_camera, images):
        """Distance map of one reference fisheye image (python/depth_estimation.py:137-203).
        ``reference_image`` and ``images`` are the [1, 3, 1, rows, cols] views of HWC images that
        the reference builds (python/depth_estimation.py:222-223); returns [rows, cols]."""
        hwc = [im[0, :, 0].permute(1, 2, 0) for im in images]
        ref_hwc = reference_image[0, :, 0].permute(1, 2, 0)
        reference = next((i for i, im in enumerate(hwc) if im.data_ptr() == ref_hwc.data_ptr()), None)
        if reference is None or reference not in self.references_indices:
            raise ValueError("reference_image must be one of `images` and a reference camera")
        slot = self.references_indices.index(reference)
        cols, rows = self.matching_resolution
        self._validate_images(hwc, (rows, cols, 3), "images")
        N.require(guide, "guide", torch.uint8, (rows, cols, 3), self.device)
        out = torch.empty([rows, cols], device=self.device)
        return self._distance(slot, reference, guide, hwc, out)

    def estimate_RGBD_panorama(self, images_to_match, images_to_stitch):
        """Distance on every reference fisheye image, then a disparity-aware stitch.

        Args:
            images_to_match: [cameras][matching_rows, matching_cols, 3] float32 in [0, 255]
            images_to_stitch: [references][rgb_stitching_rows, rgb_stitching_cols, 3] float32
                in [0, 255]
        Returns:
            rgb: [rows, cols, 3] uint8 colour panorama; distance: [rows, cols] float32 distance
            panorama (both alias the stitcher's buffers and are overwritten by the next call)
        """
        cols, rows = self.matching_resolution
        st = self.fishey_stitcher
        if self.cost_storage != "fp32":
            match = torch.stack(list(images_to_match))[None]
            stitch = torch.stack(list(images_to_stitch))[None]
            rgb, distance = self.pipeline().run(match, stitch)
            return rgb[0], distance[0]
        if len(images_to_match) != len(self.calibrations):
            raise ValueError(f"expected {len(self.calibrations)} images to match")
        if len(images_to_stitch) != len(self.references_indices):
            raise ValueError(f"expected {len(self.references_indices)} images to stitch")
        self._validate_images(images_to_match, (rows, cols, 3), "images_to_match")
        self._validate_images(images_to_stitch, (st.image_rows, st.image_cols, 3), "images_to_stitch")
        for slot, reference in enumerate(self.references_indices):
            rgb_to_guide(images_to_match[reference], self._guide)
            self._distance(slot, reference, self._guide, images_to_match, st.distances_list[slot])
        for slot, image in enumerate(images_to_stitch):
            st.images_to_stitch_list[slot].copy_(image)  # float -> uint8 truncation (depth_estimation.py:239-240)
        return st.stitch(st.images_to_stitch_list, st.distances_list)

    def estimate_RGBD_panoramas(self, images_to_match, images_to_stitch=None):
        """Batched ``estimate_RGBD_panorama`` (no counterpart in the reference, which takes one
        frame per call) on the 16-bit pipeline.

        Args:
            images_to_match: [frames, cameras, matching_rows, matching_cols, 3] float32 in [0, 255],
                or uint8 (the 8-bit images the float inputs are made from); uint8 images of another
                size (the decoded images) are resized to the matching resolution as they are staged
            images_to_stitch: [frames, references, rgb_stitching_rows, rgb_stitching_cols, 3]
                float32 in [0, 255], or uint8; None when images_to_match are the decoded uint8
                images at the stitch resolution (their references' images are stitched)
        Returns:
            rgb: [frames, rows, cols, 3] uint8, distance: [frames, rows, cols] float32 (views of
            the pipeline's buffers, overwritten by the next call)
        """
        return self.pipeline().run(images_to_match, images_to_stitch)

    @property
    def batch_distance_maps(self):
        """Filtered per-reference distance maps of the last batch, [frames, references, rows, cols]."""
        return self.pipeline().distance

    @property
    def batch_index_maps(self):
        """Selected candidate indices of the last batch, [frames, references, rows, cols]."""
        p = self.pipeline()
        return p.index.view(p.max_frames, p.R, p.rows, p.cols)

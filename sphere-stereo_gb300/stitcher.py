"""Stitcher: RGB-D panorama from RGB-D fisheye images (python/stitcher.py:35-220), same
constructor and ``stitch`` contract, running the sm_103a kernels of csrc/ssg_stitch.cu.

Tables are built once at construction (inpainting directions, blending lookup table, smoothed
and normalised blending weights); ``stitch`` reprojects each distance map to the panorama
viewpoint with a z-buffer, fills its holes and merges colour and distance.  The outputs alias
this object's buffers and are overwritten by the next call, as in the reference.
"""
from __future__ import annotations

import torch

from . import _native as N
from .utils import _cpu32, intrinsics_struct


def vectorize_calibration(calibration, device):
    """Intrinsics as the float vector of the kernels' Intrinsics struct
    [fx * s, fy * s, cx * s, cy * s, xi, alpha] (python/stitcher.py:35-46)."""
    v = torch.zeros([6], device=device)
    v[0:2] = calibration.fl * calibration.matching_scale
    v[2:4] = calibration.principal * calibration.matching_scale
    v[4] = calibration.xi
    v[5] = calibration.alpha
    return v


class Stitcher:
    def __init__(self, calibrations, reprojection_viewpoint, masks, min_dist, max_dist, matching_resolution,
                 rgb_to_stitch_resolution, panorama_resolution, device, smoothing_radius=15,
                 inpainting_iterations=32):
        """Allocate intermediate arrays and compute the stitching tables.

        Args:
            calibrations: [references] double-sphere calibrations of the cameras to stitch
            reprojection_viewpoint: [3] viewpoint of the output panorama
            masks: [references][1, matching_rows, matching_cols] valid areas (1 = reliable)
            min_dist, max_dist: distance range of the distance maps
            matching_resolution: (cols, rows) of the distance maps
            rgb_to_stitch_resolution: (cols, rows) of the colour images sampled while stitching
            panorama_resolution: (cols, rows) of the output panorama
            device: CUDA device
            smoothing_radius: radius of the box filter applied to masks and blending weights
            inpainting_iterations: hole-filling steps (should exceed the widest occlusion)
        """
        device = torch.device(device)
        if device.type != "cuda":
            raise ValueError(f"Stitcher runs on a CUDA device, got {device}; there is no CPU path")
        N.library()
        if not 1 <= len(calibrations) <= N.MAX_REFERENCES:
            raise ValueError(f"between 1 and {N.MAX_REFERENCES} references are supported")
        self.device = device
        self.min_dist = float(min_dist)
        self.max_dist = float(max_dist)
        self.inpainting_iterations = int(inpainting_iterations)
        self.cols, self.rows = matching_resolution
        self.image_cols, self.image_rows = rgb_to_stitch_resolution
        self.pano_cols, self.pano_rows = panorama_resolution
        R = len(calibrations)
        self.reference_count = R
        H, W, Hp, Wp = self.rows, self.cols, self.pano_rows, self.pano_cols

        self.reprojected_distances = torch.zeros([R, H, W], device=device)
        self.distances_stacked = torch.zeros([R, H, W], device=device)
        self.images_to_stitch = torch.zeros([R, self.image_rows, self.image_cols, 3], dtype=torch.uint8,
                                            device=device)
        self.reprojected_distances_list = [self.reprojected_distances[i] for i in range(R)]
        self.distances_list = [self.distances_stacked[i] for i in range(R)]
        self.images_to_stitch_list = [self.images_to_stitch[i] for i in range(R)]
        self.inpainting_weights_list = [torch.zeros([H, W, 2], dtype=torch.uint8, device=device) for _ in range(R)]
        self.inpainting_scratch = torch.empty([H, W], device=device)
        self.blending_sampling = torch.zeros([R, Hp, Wp, 2], device=device)
        self.blending_weights = torch.zeros([R, Hp, Wp], device=device)
        self.RGB_panorama = torch.zeros([Hp, Wp, 3], dtype=torch.uint8, device=device)
        self.distance_panorama = torch.zeros([Hp, Wp], device=device)

        # tables (python/stitcher.py:126-164); small matrices on the CPU in float32
        self.intrinsics = [intrinsics_struct(c) for c in calibrations]
        self.calibration_vectors_list = [vectorize_calibration(c, device) for c in calibrations]
        self.calibration_vectors = torch.cat(self.calibration_vectors_list).contiguous()
        self._intr = N.intrinsics_array(self.intrinsics)
        self.smoothing_radius = int(smoothing_radius)
        stream = torch.cuda.current_stream(device).cuda_stream
        # the smoothed masks depend on the masks only: kept for rig updates
        mask_stack = torch.stack([torch.as_tensor(m, dtype=torch.float32).reshape(H, W) for m in masks]).to(device)
        mask_stack = mask_stack.contiguous()
        self.smoothed_masks = torch.empty_like(mask_stack)
        N.call("ssg_box_filter", mask_stack.data_ptr(), R, H, W, self.smoothing_radius, 1.0,
               self.smoothed_masks.data_ptr(), stream)
        self._raw_weights = torch.empty_like(self.blending_weights)
        self._build_tables(calibrations, reprojection_viewpoint, stream)

    def _build_tables(self, calibrations, reprojection_viewpoint, stream: int) -> None:
        """The tables that depend on the references' poses and the viewpoint: translations,
        inpainting tables, blending LUT and weights (python/stitcher.py:126-164)."""
        H, W, Hp, Wp = self.rows, self.cols, self.pano_rows, self.pano_cols
        R = self.reference_count
        vp = torch.cat([_cpu32(reprojection_viewpoint), torch.ones(1)])
        translations = [torch.matmul(torch.inverse(_cpu32(c.rt)), vp)[:3] for c in calibrations]
        self.translations_host = torch.cat(translations).contiguous()
        if hasattr(self, "translations"):
            self.translations.copy_(self.translations_host)
        else:
            self.translations = self.translations_host.to(self.device)
        self.translations_list = [self.translations[3 * i:3 * i + 3] for i in range(R)]
        rotations = torch.cat([torch.inverse(_cpu32(c.rt)[:3, :3]) for c in calibrations]).contiguous()
        self._trans = N.floats(self.translations_host.tolist())
        for r, table in enumerate(self.inpainting_weights_list):
            N.call("ssg_inpainting_table", W, H, N.intrinsics_array([self.intrinsics[r]]),
                   N.floats(translations[r].tolist()), self.min_dist, self.max_dist, table.data_ptr(), stream)
        N.call("ssg_blending_lut", W, H, Wp, Hp, R, self._intr, N.floats(rotations.reshape(-1).tolist()), self._trans,
               self.smoothed_masks.data_ptr(), self.min_dist, self.max_dist, self.blending_sampling.data_ptr(),
               self._raw_weights.data_ptr(), stream)
        N.call("ssg_box_filter", self._raw_weights.data_ptr(), R, Hp, Wp, self.smoothing_radius, 0.0,
               self.blending_weights.data_ptr(), stream)
        N.call("ssg_normalize_weights", self.blending_weights.data_ptr(), R, Hp * Wp, stream)

    def update_extrinsics(self, calibrations, reprojection_viewpoint) -> None:
        """Rebuilds the pose-dependent tables in place after the references' extrinsics (``rt``)
        or the viewpoint changed (calibration refinement; no counterpart in the reference, which
        builds them once in its constructor).  Intrinsics, resolutions and masks stay; buffers
        keep their addresses.  The result equals a Stitcher constructed with the new poses."""
        if len(calibrations) != self.reference_count:
            raise ValueError(f"expected {self.reference_count} calibrations, got {len(calibrations)}")
        def fields(k):
            return tuple(getattr(k, f) for f, _ in k._fields_)

        for c, k in zip(calibrations, self.intrinsics):
            if fields(intrinsics_struct(c)) != fields(k):
                raise ValueError("update_extrinsics keeps the intrinsics; construct a new Stitcher to change them")
        self._build_tables(calibrations, reprojection_viewpoint, torch.cuda.current_stream(self.device).cuda_stream)

    def reproject_and_inpaint(self, reference: int, distance_map: torch.Tensor) -> None:
        """Reprojected, hole-filled distance map of one reference (python/stitcher.py:184-200)
        into ``self.reprojected_distances[reference]``."""
        out = self.reprojected_distances_list[reference]
        stream = N.stream_of(distance_map)
        N.call("ssg_reproject_distance", distance_map.data_ptr(), out.data_ptr(), self.cols, self.rows,
               N.intrinsics_array([self.intrinsics[reference]]),
               N.floats(self.translations_host[3 * reference:3 * reference + 3].tolist()), 1, stream)
        N.call("ssg_inpaint", out.data_ptr(), self.inpainting_weights_list[reference].data_ptr(),
               self.inpainting_scratch.data_ptr(), self.cols, self.rows, self.max_dist, self.inpainting_iterations,
               stream)

    def merge(self) -> None:
        """Blend the stacked maps and images into the panorama (python/stitcher.py:205-218)."""
        N.call("ssg_merge_panorama", self.blending_sampling.data_ptr(), self.blending_weights.data_ptr(),
               self.reprojected_distances.data_ptr(), self.distances_stacked.data_ptr(),
               self.images_to_stitch.data_ptr(), self.image_rows, self.image_cols, self._trans, self._intr,
               self.reference_count, self.cols, self.rows, self.pano_cols, self.pano_rows,
               self.distance_panorama.data_ptr(), self.RGB_panorama.data_ptr(),
               N.stream_of(self.distance_panorama))

    def stitch(self, images, distance_maps):
        """Stitch colour images and distance maps into an RGB-D panorama.

        Args:
            images: [references][rgb_to_stitch_rows, rgb_to_stitch_cols, 3] uint8
            distance_maps: [references][matching_rows, matching_cols] float32
        Returns:
            rgb: [rows, cols, 3] uint8 colour panorama, distance: [rows, cols] float32
            (both alias this object's buffers)
        """
        if len(images) != self.reference_count or len(distance_maps) != self.reference_count:
            raise ValueError(f"expected {self.reference_count} images and distance maps")
        for r, (image, distance_map) in enumerate(zip(images, distance_maps)):
            N.require(image, f"images[{r}]", torch.uint8, (self.image_rows, self.image_cols, 3), self.device)
            N.require(distance_map, f"distance_maps[{r}]", torch.float32, (self.rows, self.cols), self.device)
            self.reproject_and_inpaint(r, distance_map)
            if image.data_ptr() != self.images_to_stitch_list[r].data_ptr():
                self.images_to_stitch_list[r].copy_(image)
            if distance_map.data_ptr() != self.distances_list[r].data_ptr():
                self.distances_list[r].copy_(distance_map)
        self.merge()
        return self.RGB_panorama, self.distance_panorama

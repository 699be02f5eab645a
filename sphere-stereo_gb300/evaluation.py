"""Evaluation of RGB-D panoramas against ground truth on the GPU: the metrics of
evaluate_rgbd_panorama (python/utils.py:206-250) -- PSNR and SSIM of the colour panorama, MAE,
RMSE and bad-pixel ratios of the inverse-distance panorama -- reduced on the device for a batch
of frames (ssg_eval_panoramas).

The definitions are scikit-image's peak_signal_noise_ratio(gt, est) and
structural_similarity(gt, est, multichannel=True) on x / 255 float32 images, as the reference
calls them, and the reference's numpy expressions for the distance errors; the C ABI's
documentation gives the arithmetic.
"""
from __future__ import annotations

import os

import numpy as np
import torch

from . import _native as N
from . import imageio

METRICS = ("psnr", "ssim", "mae", "rmse")


def _batched(t: torch.Tensor, name: str, dtype: torch.dtype, channels: int | None) -> torch.Tensor:
    want = 3 if channels is None else 4
    if t.dim() == want - 1:
        t = t.unsqueeze(0)
    if t.dim() != want:
        raise ValueError(f"{name} must be [frames,] rows, cols{', 3' if channels else ''} (got {tuple(t.shape)})")
    N.require(t, name, dtype)
    return t


def evaluate_panoramas(rgb: torch.Tensor, inv_distance: torch.Tensor, gt_rgb: torch.Tensor,
                       gt_inv_distance: torch.Tensor, bad_px_ratio_thresholds=()) -> torch.Tensor:
    """Metrics of a batch of panoramas on their device.

    Args:
        rgb, gt_rgb: uint8 [frames, rows, cols, 3] (or one frame [rows, cols, 3]), CUDA
        inv_distance, gt_inv_distance: float32 [frames, rows, cols] (or [rows, cols]), CUDA
        bad_px_ratio_thresholds: up to 16 thresholds on |inv_distance - gt_inv_distance|
    Returns:
        float64 [frames, 4 + thresholds] on the device: psnr, ssim, mae, rmse, then the bad-pixel
        ratios in percent.
    """
    rgb = _batched(rgb, "rgb", torch.uint8, 3)
    gt_rgb = _batched(gt_rgb, "gt_rgb", torch.uint8, 3)
    inv_distance = _batched(inv_distance, "inv_distance", torch.float32, None)
    gt_inv_distance = _batched(gt_inv_distance, "gt_inv_distance", torch.float32, None)
    frames, rows, cols = rgb.shape[:3]
    for t, name in ((gt_rgb, "gt_rgb"), (inv_distance, "inv_distance"), (gt_inv_distance, "gt_inv_distance")):
        if tuple(t.shape[:3]) != (frames, rows, cols):
            raise ValueError(f"{name} has shape {tuple(t.shape)}, rgb {tuple(rgb.shape)}")
        if t.device != rgb.device:
            raise ValueError(f"{name} is on {t.device}, rgb on {rgb.device}")
    thresholds = [float(t) for t in bad_px_ratio_thresholds]
    k = len(thresholds)
    if k > N.SSG_EVAL_MAX_THRESHOLDS:
        raise ValueError(f"at most {N.SSG_EVAL_MAX_THRESHOLDS} thresholds (got {k})")
    scratch_bytes = N.library().ssg_eval_scratch_bytes(frames, k)
    scratch = torch.empty(max(1, scratch_bytes // 8), dtype=torch.float64, device=rgb.device)
    out = torch.empty((frames, 4 + k), dtype=torch.float64, device=rgb.device)
    with torch.cuda.device(rgb.device):
        N.call("ssg_eval_panoramas", cols, rows, frames, rgb.data_ptr(), gt_rgb.data_ptr(), inv_distance.data_ptr(),
               gt_inv_distance.data_ptr(), N.floats(thresholds) if k else None, k, scratch.data_ptr(),
               out.data_ptr(), N.stream_of(rgb))
    return out


def metrics_dict(row, thresholds_count: int) -> dict:
    """The reference's result dict (python/utils.py:246) from one row of evaluate_panoramas."""
    v = [float(x) for x in row]
    return {"ssim": v[1], "psnr": v[0], "mae": v[2], "rmse": v[3], "bad_px_ratios": v[4:4 + thresholds_count]}


def evaluate_rgbd_panorama_tensors(rgb, inv_distance, gt_rgb, gt_inv_distance, bad_px_ratio_thresholds) -> dict:
    """One panorama already in memory: the dict evaluate_rgbd_panorama returns."""
    out = evaluate_panoramas(rgb, inv_distance, gt_rgb, gt_inv_distance, bad_px_ratio_thresholds)
    return metrics_dict(out[0].cpu(), len(bad_px_ratio_thresholds))


def evaluate_rgbd_panorama(rgbd_panoramas, filename, dataset_path, bad_px_ratio_thresholds, panorama_resolution,
                           device="cuda"):
    """python/utils.py:206-250, same arguments and result: reads gt/rgb_<name>.png and
    gt/inv_distance_<name>.exr under dataset_path (imageio readers), brings them to
    panorama_resolution (cols, rows) with the linear resize of the input path
    (utils.resize_linear, the effective interpolation of the reference's cv2.resize call), and
    evaluates rgbd_panoramas[filename] on `device`.  Returns None (with a warning) where the
    reference does: unknown frame, missing or mistyped ground truth."""
    import warnings

    from . import utils

    try:
        pano = rgbd_panoramas[filename]
    except KeyError:
        warnings.warn("Invalid ground truth for file " + filename)
        return None
    read_name = os.path.splitext(filename)[0]
    gt_rgb = imageio.imread(os.path.join(dataset_path, "gt/rgb_" + read_name + ".png"))
    gt_distance = imageio.imread(os.path.join(dataset_path, "gt/inv_distance_" + read_name + ".exr"))
    est_rgb = _tensor(pano["rgb"], device)
    est_inv = _tensor(pano["inv_distance"], device)
    if (gt_rgb is None or gt_distance is None or gt_rgb.dtype != np.uint8 or gt_distance.dtype != np.float32
            or est_rgb.dtype != torch.uint8 or est_inv.dtype != torch.float32 or gt_rgb.ndim != 3
            or gt_distance.ndim != 2):
        warnings.warn("Invalid ground truth for file " + filename + ". Will be ignored for evaluation")
        return None
    cols, rows = int(panorama_resolution[0]), int(panorama_resolution[1])
    gt_rgb_t = torch.as_tensor(np.ascontiguousarray(gt_rgb), device=device)
    gt_inv_t = torch.as_tensor(np.ascontiguousarray(gt_distance), device=device)
    if tuple(gt_rgb_t.shape[:2]) != (rows, cols):
        gt_rgb_t = utils.resize_linear(gt_rgb_t, (cols, rows), out_dtype=torch.uint8)
    if tuple(gt_inv_t.shape) != (rows, cols):
        gt_inv_t = utils.resize_linear(gt_inv_t.unsqueeze(-1), (cols, rows))[..., 0].contiguous()
    return evaluate_rgbd_panorama_tensors(est_rgb, est_inv, gt_rgb_t, gt_inv_t, bad_px_ratio_thresholds)


def _tensor(a, device) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.to(device).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), device=device)

"""Calibration container and parser, double-sphere helpers and the guide colour transform:
the public helpers of the reference's python/utils.py:40-155, same names and arguments.

``unproject``, ``project`` and ``rgb2yCbCr`` are the reference's helper functions (torch
expressions, any device); the per-frame path does not call them, it runs the same model inside
the CUDA kernels.  The helpers below this module's public API turn calibrations into the
argument structs of the C ABI.
"""
from __future__ import annotations

import math

import torch

from . import _native as N


class Calibration:
    def __init__(self, original_resolution, principal, fl, xi, alpha, rt, matching_scale):
        """Double-sphere intrinsics (python/utils.py:40-55).

        Args:
            original_resolution, principal, fl, xi, alpha: double-sphere intrinsics at the
                original (cols, rows) resolution
            rt: [4, 4] camera pose, camera -> rig
            matching_scale: [2] scale applied to the resolution, principal point and focal length
                when working with images resized to the matching resolution
        """
        self.original_resolution = original_resolution
        self.principal = principal
        self.fl = fl
        self.xi = xi
        self.alpha = alpha
        self.rt = rt
        self.matching_scale = matching_scale


def unproject(uv, calib):
    """Pixels -> unit sphere, double-sphere model (python/utils.py:57-73), scaled by
    calib.matching_scale.  Returns (points [..., 3], valid [...])."""
    m_xy = (uv - calib.principal * calib.matching_scale) / (calib.fl * calib.matching_scale)
    r2 = torch.sum(m_xy ** 2, dim=-1, keepdim=True)
    m_z = ((1 - calib.alpha ** 2 * r2)
           / (calib.alpha * torch.sqrt(torch.clamp(1 - (2 * calib.alpha - 1) * r2, min=0)) + 1 - calib.alpha))
    point = torch.cat([m_xy, m_z], dim=-1)
    point = ((m_z * calib.xi + torch.sqrt(m_z ** 2 + (1 - calib.xi ** 2) * r2)) / (m_z ** 2 + r2)) * point
    point[..., 2] -= calib.xi
    valid = 1 - (2 * calib.alpha - 1) * r2 >= 0
    return point, valid[..., 0]


def project(point, calib):
    """Points -> pixels, double-sphere model (python/utils.py:75-94), scaled by
    calib.matching_scale.  Returns (uv [..., 2], valid [...])."""
    d1 = torch.norm(point, dim=-1, keepdim=True)
    c = calib.xi * d1 + point[..., 2:3]
    d2 = torch.norm(torch.cat([point[..., :2], c], dim=-1), dim=-1, keepdim=True)
    norm = calib.alpha * d2 + (1 - calib.alpha) * c
    w1 = (1 - calib.alpha) / calib.alpha if calib.alpha > 0.5 else calib.alpha / (1 - calib.alpha)
    w2 = (w1 + calib.xi) / math.sqrt(2 * w1 * calib.xi + calib.xi ** 2 + 1)
    valid = point[..., 2:3] > -w2 * d1
    uv = (calib.fl * calib.matching_scale * point[..., :2]) / norm + calib.principal * calib.matching_scale
    return uv, valid[..., 0]


def parse_json_calib(raw_calibration, matching_resolution, device):
    """Basalt calibration (the ``value0`` dictionary) -> list of Calibration
    (python/utils.py:96-142).  Raises for any camera model other than double sphere."""
    from scipy.spatial.transform import Rotation

    calibrations = []
    for extrinsics, intrinsics, original_resolution in zip(raw_calibration["T_imu_cam"],
                                                           raw_calibration["intrinsics"],
                                                           raw_calibration["resolution"]):
        if intrinsics["camera_type"] != "ds":
            raise Exception("Unexpected camera model. The current implementation only support double sphere.")
        ci = intrinsics["intrinsics"]
        r = Rotation.from_quat([extrinsics["qx"], extrinsics["qy"], extrinsics["qz"], extrinsics["qw"]])
        t = torch.tensor([extrinsics["px"], extrinsics["py"], extrinsics["pz"]], device=device)
        rt = torch.eye(4, device=device)
        rt[:3, :3] = torch.tensor(r.as_matrix(), device=device)
        rt[:3, 3] = t
        calibrations.append(Calibration(
            original_resolution,
            torch.tensor([ci["cx"], ci["cy"]], device=device),
            torch.tensor([ci["fx"], ci["fy"]], device=device),
            ci["xi"], ci["alpha"], rt,
            torch.tensor([matching_resolution[0] / original_resolution[0],
                          matching_resolution[1] / original_resolution[1]], device=device)))
    return calibrations


def rgb2yCbCr(rgb):
    """Fixed-coefficient YCbCr with clamps (python/utils.py:144-155), float result.  The
    estimator uses the fused CUDA version with the uint8 cast, ``rgb_to_guide``."""
    rgb = rgb.float()
    yuv = torch.zeros_like(rgb)
    yuv[:, :, 0] = torch.clamp(16 + 0.1826 * rgb[:, :, 0] + 0.6142 * rgb[:, :, 1] + 0.062 * rgb[:, :, 2],
                               min=16, max=235)
    yuv[:, :, 1] = torch.clamp(128 - 0.1006 * rgb[:, :, 0] - 0.3386 * rgb[:, :, 1] + 0.4392 * rgb[:, :, 2],
                               min=16, max=240)
    yuv[:, :, 2] = torch.clamp(128 + 0.4392 * rgb[:, :, 0] - 0.3989 * rgb[:, :, 1] - 0.0403 * rgb[:, :, 2],
                               min=16, max=240)
    return yuv


def rgb_to_guide(rgb: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """``rgb2yCbCr(rgb).type(torch.uint8)`` (python/depth_estimation.py:227) in one CUDA kernel.
    rgb: [rows, cols, 3] float32 CUDA tensor."""
    N.require(rgb, "rgb", torch.float32)
    if rgb.dim() != 3 or rgb.shape[-1] != 3:
        raise ValueError("rgb must be [rows, cols, 3]")
    if out is None:
        out = torch.empty(rgb.shape, dtype=torch.uint8, device=rgb.device)
    N.require(out, "out", torch.uint8, tuple(rgb.shape), rgb.device)
    N.call("ssg_rgb_to_guide", rgb.data_ptr(), rgb.numel() // 3, out.data_ptr(), N.stream_of(rgb))
    return out


def resize_linear(images: torch.Tensor, size, out_dtype: torch.dtype = torch.float32) -> torch.Tensor:
    """The linear resize of the reference's input path (python/utils.py:198-201, cv2.resize with
    the default INTER_LINEAR in effect) on the GPU: ssg_resize_linear.

    Args:
        images: [rows, cols, channels] or [images, rows, cols, channels] uint8 or float32 CUDA tensor
            (channels 1..4)
        size: (cols, rows) of the result
        out_dtype: torch.float32 (uint8 inputs are converted as the reference's astype(float32)
            does, then resized) or torch.uint8 (uint8 inputs only: OpenCV's fixed-point path)
    """
    single = images.dim() == 3
    x = images.unsqueeze(0) if single else images
    if x.dim() != 4 or not 1 <= x.shape[-1] <= 4:
        raise ValueError(f"images must be [images,] rows, cols, channels (got {tuple(images.shape)})")
    if x.dtype not in (torch.uint8, torch.float32):
        raise TypeError(f"images must be uint8 or float32 (got {x.dtype})")
    N.require(x, "images", x.dtype)
    cols, rows = int(size[0]), int(size[1])
    src_type = N.PIXEL_U8 if x.dtype == torch.uint8 else N.PIXEL_F32
    dst_type = N.PIXEL_U8 if out_dtype == torch.uint8 else N.PIXEL_F32
    out = torch.empty((x.shape[0], rows, cols, x.shape[-1]), dtype=out_dtype, device=x.device)
    with torch.cuda.device(x.device):
        N.call("ssg_resize_linear", x.data_ptr(), src_type, x.shape[2], x.shape[1], x.shape[3], out.data_ptr(),
               dst_type, cols, rows, x.shape[0], N.stream_of(x))
    return out[0] if single else out


def read_input_images(filename, dataset_path, matching_resolution, rgb_to_stitch_resolution, calibrations,
                      references_indices, device="cuda"):
    """python/utils.py:157-204 with the resize on the GPU: reads <dataset_path>/cam<i>/<filename>
    (PNG or EXR: imageio.imread), maps uint8 to float32, uint16 to float32 / 255 and float32 to
    255 * clip(x, 0, 1) (with the reference's warnings), and resizes to the matching resolution
    (every camera) and the stitching resolution (reference cameras).  Returns the reference's dict
    with lists of float32 [rows, cols, 3] CUDA tensors."""
    import os
    import warnings

    import numpy as np

    from . import imageio

    images_to_match, images_to_stitch = [], []
    valid_frame = True
    for cam_index, calibration in enumerate(calibrations):
        file_path = os.path.join(dataset_path, "cam" + str(cam_index)) + "/" + filename
        image = imageio.imread(file_path)
        if image is not None:
            res = calibration.original_resolution
            if image.shape == (res[1], res[0], 3):
                if image.dtype == np.uint8:
                    t = torch.as_tensor(np.ascontiguousarray(image), device=device)  # uint8 upload
                elif image.dtype == np.uint16:
                    t = torch.as_tensor(image.astype(np.float32) / 255, device=device)
                elif image.dtype == np.float32:
                    if np.max(image) > 1:
                        image = np.clip(image, 0, 1)
                        warnings.warn("Image has out-of-range float values for file " + file_path
                                      + ". Clipped for processing.")
                    t = torch.as_tensor(np.ascontiguousarray(image * 255), device=device)
                else:
                    warnings.warn("Invalide image type for file " + file_path)
                    valid_frame = False
            else:
                warnings.warn("Invalid image size / channels for file " + file_path)
                valid_frame = False
        else:
            warnings.warn("Cannot read image for file " + file_path)
            valid_frame = False
        if valid_frame:
            if cam_index in references_indices:
                images_to_stitch.append(resize_linear(t, rgb_to_stitch_resolution))
            images_to_match.append(resize_linear(t, matching_resolution))
    return {"images_to_match": images_to_match, "images_to_stitch": images_to_stitch, "is_valid": valid_frame}


# ---------------------------------------------------------------------------------------------
# Calibration -> C ABI structs.  Small matrices are computed on the CPU in float32 with the
# reference's own expressions, so that every device and every run sees the same values.
# ---------------------------------------------------------------------------------------------

def _cpu32(t) -> torch.Tensor:
    return torch.as_tensor(t).detach().to("cpu", torch.float32)


def camera_struct(calib: Calibration) -> N.ssg_camera:
    """{fl * matching_scale, principal * matching_scale} in float32 plus xi, alpha as doubles."""
    fs = _cpu32(calib.fl) * _cpu32(calib.matching_scale)
    ps = _cpu32(calib.principal) * _cpu32(calib.matching_scale)
    return N.ssg_camera(float(fs[0]), float(fs[1]), float(ps[0]), float(ps[1]), float(calib.xi), float(calib.alpha))


def intrinsics_struct(calib: Calibration) -> N.ssg_intrinsics:
    """vectorize_calibration (python/stitcher.py:35-46) as the C struct."""
    fs = _cpu32(calib.fl) * _cpu32(calib.matching_scale)
    ps = _cpu32(calib.principal) * _cpu32(calib.matching_scale)
    return N.ssg_intrinsics(float(fs[0]), float(fs[1]), float(ps[0]), float(ps[1]),
                            float(torch.tensor(calib.xi, dtype=torch.float32)),
                            float(torch.tensor(calib.alpha, dtype=torch.float32)))


def relative_poses(calibrations, reference_index: int) -> list[float]:
    """Rows 0..2 of inverse(camera.rt) @ reference.rt for every camera
    (python/depth_estimation.py:104, :156), flattened: camera_count x 12 floats."""
    ref_rt = _cpu32(calibrations[reference_index].rt)
    out = []
    for c in calibrations:
        rt = torch.matmul(torch.inverse(_cpu32(c.rt)), ref_rt)
        out.extend(rt[:3].reshape(12).tolist())
    return out

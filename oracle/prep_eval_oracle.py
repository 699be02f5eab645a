"""TEST INFRASTRUCTURE -- CPU oracle of the input resize and of the evaluation metrics.  Used only
by tests/ as the checker; the product package never imports it.

resize_linear: OpenCV's linear resize (the interpolation the reference's cv2.resize call in
python/utils.py:198-201 performs, INTER_LINEAR being the default in effect), restated from its
published algorithm in numpy float32 arithmetic -- the same statements the device kernel
follows (pixel-centre mapping computed in double and rounded to float32, clamped taps,
separately rounded products and sums; 2x2 averages for an exact 2x reduction; 11-bit fixed-point
weights for uint8 -> uint8).  cv2 is absent here, so the restatement is not pinned against
OpenCV's own outputs (parity unpinned for this row).

evaluate: python/utils.py:224-244 -- scikit-image 0.18's peak_signal_noise_ratio and
structural_similarity(multichannel=True) restated with numpy and scipy.ndimage.uniform_filter
(the filter scikit-image uses), and the reference's numpy expressions for MAE, RMSE and bad-pixel
ratios.  scikit-image is absent here; the statements follow its published source.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.ndimage import uniform_filter


# --------------------------------------------------------------------------------------------
# resize
# --------------------------------------------------------------------------------------------
def _column_taps(src: int, dst: int):
    scale = 1.0 / (dst / src)
    fx = ((np.arange(dst, dtype=np.float64) + 0.5) * scale - 0.5).astype(np.float32)
    sx = np.floor(fx).astype(np.int64)
    fx = (fx - sx.astype(np.float32)).astype(np.float32)
    low = sx < 0
    fx[low], sx[low] = 0.0, 0
    high = sx >= src - 1
    fx[high], sx[high] = 0.0, src - 1
    return sx, np.minimum(sx + 1, src - 1), fx


def _row_taps(src: int, dst: int):
    scale = 1.0 / (dst / src)
    fy = ((np.arange(dst, dtype=np.float64) + 0.5) * scale - 0.5).astype(np.float32)
    sy = np.floor(fy).astype(np.int64)
    fy = (fy - sy.astype(np.float32)).astype(np.float32)
    return np.clip(sy, 0, src - 1), np.clip(sy + 1, 0, src - 1), fy


def _fixed(f: np.ndarray) -> np.ndarray:
    w = (np.float32(1.0) - f).astype(np.float32) * np.float32(2048.0)
    return np.clip(np.rint(w), -32768, 32767).astype(np.int64)


def resize_linear(img: np.ndarray, size, out_dtype=np.float32) -> np.ndarray:
    """img: [rows, cols, channels] uint8 or float32; size (cols, rows).  The result is C-contiguous
    (row-major, like cv2.resize's): the fancy indexing below yields a transposed layout, which
    torch.tensor would keep, and the reference hands its tensors' raw memory to its kernels."""
    return np.ascontiguousarray(_resize_linear(img, size, out_dtype))


def _resize_linear(img: np.ndarray, size, out_dtype=np.float32) -> np.ndarray:
    src = np.asarray(img)
    rows_in, cols_in = src.shape[:2]
    cols, rows = int(size[0]), int(size[1])
    if cols_in == 2 * cols and rows_in == 2 * rows:
        a, b = src[0::2, 0::2], src[0::2, 1::2]
        c, d = src[1::2, 0::2], src[1::2, 1::2]
        if out_dtype == np.uint8:
            s = a.astype(np.int64) + b + c + d
            return ((s + 2) >> 2).astype(np.uint8)
        f = [x.astype(np.float32) for x in (a, b, c, d)]
        return (((f[0] + f[1]) + f[2]) + f[3]) * np.float32(0.25)
    x0, x1, fx = _column_taps(cols_in, cols)
    y0, y1, fy = _row_taps(rows_in, rows)
    if out_dtype == np.uint8:
        a0 = _fixed(fx)[None, :, None]
        a1 = 2048 - a0
        b0 = _fixed(fy)[:, None, None]
        b1 = 2048 - b0
        s = src.astype(np.int64)
        h0 = s[y0][:, x0] * a0 + s[y0][:, x1] * a1
        h1 = s[y1][:, x0] * a0 + s[y1][:, x1] * a1
        v = (h0 * b0 + h1 * b1 + (1 << 21)) >> 22
        return np.clip(v, 0, 255).astype(np.uint8)
    s = src.astype(np.float32)
    a0 = (np.float32(1.0) - fx).astype(np.float32)[None, :, None]
    a1 = fx[None, :, None]
    b0 = (np.float32(1.0) - fy).astype(np.float32)[:, None, None]
    b1 = fy[:, None, None]
    h0 = (s[y0][:, x0] * a0).astype(np.float32) + (s[y0][:, x1] * a1).astype(np.float32)
    h1 = (s[y1][:, x0] * a0).astype(np.float32) + (s[y1][:, x1] * a1).astype(np.float32)
    return ((h0 * b0).astype(np.float32) + (h1 * b1).astype(np.float32)).astype(np.float32)


# --------------------------------------------------------------------------------------------
# evaluation
# --------------------------------------------------------------------------------------------
def psnr(gt_rgb: np.ndarray, rgb: np.ndarray) -> float:
    """peak_signal_noise_ratio(gt / 255, est / 255) on float32 images: data range 1 (float
    images, no negative value), mse in float64 over float32 squared differences."""
    a = gt_rgb.astype(np.float32) / 255
    b = rgb.astype(np.float32) / 255
    d = (a - b).astype(np.float32)
    mse = np.mean((d * d).astype(np.float32), dtype=np.float64)
    with np.errstate(divide="ignore"):
        return float(10 * np.log10(1.0 / mse))


def ssim(gt_rgb: np.ndarray, rgb: np.ndarray) -> float:
    """structural_similarity(gt / 255, est / 255, multichannel=True): per channel on float64
    values, 7x7 uniform windows, sample covariances, data range 2 (the float dtype range),
    K1 = 0.01, K2 = 0.03, the map cropped by 3 pixels and averaged; the mean over channels."""
    a = (gt_rgb.astype(np.float32) / 255).astype(np.float64)
    b = (rgb.astype(np.float32) / 255).astype(np.float64)
    win, np_ = 7, 49
    cov_norm = np_ / (np_ - 1)
    c1, c2 = (0.01 * 2.0) ** 2, (0.03 * 2.0) ** 2
    pad = (win - 1) // 2
    out = []
    for ch in range(a.shape[2]):
        x, y = a[:, :, ch], b[:, :, ch]
        ux = uniform_filter(x, size=win)
        uy = uniform_filter(y, size=win)
        uxx = uniform_filter(x * x, size=win)
        uyy = uniform_filter(y * y, size=win)
        uxy = uniform_filter(x * y, size=win)
        vx = cov_norm * (uxx - ux * ux)
        vy = cov_norm * (uyy - uy * uy)
        vxy = cov_norm * (uxy - ux * uy)
        a1, a2 = 2 * ux * uy + c1, 2 * vxy + c2
        b1, b2 = ux ** 2 + uy ** 2 + c1, vx + vy + c2
        s = (a1 * a2) / (b1 * b2)
        out.append(s[pad:-pad, pad:-pad].mean(dtype=np.float64))
    return float(np.mean(out))


def evaluate(rgb, inv_distance, gt_rgb, gt_inv_distance, thresholds) -> dict:
    """python/utils.py:224-246 on numpy arrays: the reference's result dict."""
    err = np.abs(inv_distance.astype(np.float32) - gt_inv_distance.astype(np.float32)).astype(np.float32)
    n = err.size
    mae = float(np.sum(err, dtype=np.float64) / n)
    err2 = (err * err).astype(np.float32)
    rmse = float(math.sqrt(np.sum(err2, dtype=np.float64) / n))
    bad = [float(100 * np.sum(err > np.float32(t)) / n) for t in thresholds]
    return {"ssim": ssim(gt_rgb, rgb), "psnr": psnr(gt_rgb, rgb), "mae": mae, "rmse": rmse, "bad_px_ratios": bad}

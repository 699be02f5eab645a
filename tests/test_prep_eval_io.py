"""Input preparation, evaluation metrics and panorama files on the CPU: the PNG / EXR codecs
(round trips, every PNG filter type, ZIP-compressed EXR blocks), the reference-shaped
save_rgbd_panorama, and the oracles of the resize and of the metrics against independent
formulations (torch's bilinear interpolation, direct window sums, closed forms)."""
from __future__ import annotations

import importlib
import os
import struct
import zlib

import numpy as np
import pytest
import torch

import prep_eval_oracle as po
from conftest import PACKAGE

io = importlib.import_module(PACKAGE + ".imageio")


def _rng(seed=7):
    return np.random.default_rng(seed)


@pytest.mark.parametrize("shape", [(5, 7), (16, 9, 3), (1, 1, 3)])
def test_png_round_trip(shape):
    a = _rng().integers(0, 256, shape, dtype=np.uint8)
    b = io.decode_png(io.encode_png(a))
    assert b.dtype == np.uint8 and b.shape == a.shape
    assert np.array_equal(a, b)


def test_png_file_holds_rgb_of_a_bgr_array(tmp_path):
    a = np.zeros((2, 3, 3), np.uint8)
    a[..., 0], a[..., 2] = 10, 200  # B, R
    data = io.encode_png(a)
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    # IHDR: width 3, height 2, depth 8, colour type 2
    assert struct.unpack(">IIBB", data[16:26]) == (3, 2, 8, 2)
    raw = zlib.decompress(data[data.index(b"IDAT") + 4:data.index(b"IEND") - 8])
    assert raw[0] == 0 and raw[1:4] == bytes([200, 0, 10])  # R, G, B in the file
    assert io.imwrite(str(tmp_path / "x.png"), a)
    assert np.array_equal(io.imread(str(tmp_path / "x.png")), a)


def _png_with_filters(img: np.ndarray, filters) -> bytes:
    """A PNG whose rows use the given filter types (encoder written from the specification)."""
    rows, cols, ch = img.shape
    stride = cols * ch
    raw = img.reshape(rows, stride).astype(np.int32)
    out = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(rows):
        f = filters[y % len(filters)]
        line = raw[y]
        left = np.concatenate([np.zeros(ch, np.int32), line[:-ch]])
        upleft = np.concatenate([np.zeros(ch, np.int32), prev[:-ch]])
        if f == 0:
            enc = line
        elif f == 1:
            enc = line - left
        elif f == 2:
            enc = line - prev
        elif f == 3:
            enc = line - (left + prev) // 2
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            enc = line - pred
        out += bytes([f]) + bytes((enc & 0xFF).astype(np.uint8))
        prev = line
    ihdr = struct.pack(">IIBBBBB", cols, rows, 8, {1: 0, 3: 2, 4: 6}[ch], 0, 0, 0)
    return b"\x89PNG\r\n\x1a\n" + io._png_chunk(b"IHDR", ihdr) + io._png_chunk(b"IDAT", zlib.compress(bytes(out))) \
        + io._png_chunk(b"IEND", b"")


@pytest.mark.parametrize("ch", [1, 3, 4])
def test_png_decoder_undoes_every_filter(ch):
    img = _rng(ch).integers(0, 256, (6, 5, ch), dtype=np.uint8)
    got = io.decode_png(_png_with_filters(img, [0, 1, 2, 3, 4]))
    want = img[:, :, 0] if ch == 1 else (img[:, :, ::-1] if ch == 3 else img[:, :, [2, 1, 0, 3]])
    assert np.array_equal(got, want)


def test_png_rejects_a_bad_crc():
    data = bytearray(io.encode_png(np.zeros((2, 2), np.uint8)))
    data[20] ^= 1
    with pytest.raises(ValueError):
        io.decode_png(bytes(data))


@pytest.mark.parametrize("shape", [(4, 6), (3, 5, 3), (1, 1)])
def test_exr_round_trip(shape, tmp_path):
    a = _rng().standard_normal(shape).astype(np.float32)
    a.flat[0] = np.inf
    b = io.decode_exr(io.encode_exr(a))
    assert b.dtype == np.float32 and b.shape == a.shape
    assert np.array_equal(a, b)
    p = str(tmp_path / "d.exr")
    io.imwrite(p, a)
    assert np.array_equal(io.imread(p), a)


def _zip_exr(image: np.ndarray, lines: int) -> bytes:
    """An OpenEXR file with ZIP(S) blocks, from the uncompressed encoder's header (compression
    byte patched) and the format's predictor and interleave, written from the specification."""
    rows, cols = image.shape
    plain = io.encode_exr(image)
    hdr_end = plain.index(b"screenWindowWidth")
    hdr_end = plain.index(b"\0", hdr_end + len("screenWindowWidth") + 1)  # end of the type name
    hdr_end += 1 + 4 + 4 + 1  # size, value, terminator
    header = bytearray(plain[:hdr_end])
    at = header.index(b"compression\0compression\0") + len("compression\0compression\0") + 4
    header[at] = 3 if lines == 16 else 2
    chunks = []
    for y in range(0, rows, lines):
        n = min(lines, rows - y)
        raw = np.ascontiguousarray(image[y:y + n], dtype="<f4").tobytes()
        b = np.frombuffer(raw, np.uint8)
        inter = np.concatenate([b[0::2], b[1::2]]).astype(np.int32)
        pred = inter.copy()
        pred[1:] = (inter[1:] - inter[:-1] + 128 + 256) & 0xFF
        chunks.append((y, zlib.compress(pred.astype(np.uint8).tobytes())))
    first = len(header) + 8 * len(chunks)
    offsets, body, pos = [], bytearray(), first
    for y, c in chunks:
        offsets.append(pos)
        body += struct.pack("<ii", y, len(c)) + c
        pos += 8 + len(c)
    return bytes(header) + struct.pack(f"<{len(offsets)}Q", *offsets) + bytes(body)


@pytest.mark.parametrize("lines", [1, 16])
def test_exr_zip_blocks(lines):
    a = (np.arange(37 * 11, dtype=np.float32).reshape(37, 11) * 0.25).astype(np.float32)
    assert np.array_equal(io.decode_exr(_zip_exr(a, lines)), a)


def test_imread_of_missing_or_foreign_files(tmp_path):
    assert io.imread(str(tmp_path / "none.png")) is None
    (tmp_path / "x.png").write_bytes(b"not an image")
    assert io.imread(str(tmp_path / "x.png")) is None


def test_save_rgbd_panorama_layout(tmp_path):
    os.makedirs(tmp_path / "output")
    rgb = _rng().integers(0, 256, (8, 16, 3), dtype=np.uint8)
    inv = _rng().random((8, 16), dtype=np.float32)
    io.save_rgbd_panorama({"12.png": {"rgb": torch.as_tensor(rgb), "inv_distance": inv}}, "12.png", str(tmp_path))
    assert np.array_equal(io.imread(str(tmp_path / "output" / "rgb_12.png")), rgb)
    assert np.array_equal(io.imread(str(tmp_path / "output" / "inv_distance_12.exr")), inv)
    io.save_rgbd_panorama({}, "13.png", str(tmp_path))  # a missing frame is ignored
    assert not os.path.exists(tmp_path / "output" / "rgb_13.png")


# --------------------------------------------------------------------------------------------
# resize oracle
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("src,dst", [((37, 29), (64, 48)), ((1216, 1216), (1024, 1024)), ((50, 40), (31, 17))])
def test_resize_oracle_matches_torch_bilinear(src, dst):
    """Pixel-centre bilinear with edge clamping is torch's align_corners=False interpolation."""
    img = _rng().random((src[1], src[0], 3), dtype=np.float32) * 255
    ours = po.resize_linear(img, dst)
    t = torch.nn.functional.interpolate(torch.as_tensor(img).permute(2, 0, 1)[None], size=(dst[1], dst[0]),
                                        mode="bilinear", align_corners=False)[0].permute(1, 2, 0).numpy()
    assert ours.shape == (dst[1], dst[0], 3) and ours.dtype == np.float32
    assert np.max(np.abs(ours - t)) < 2e-3


def test_resize_oracle_identity_and_area():
    img = _rng().integers(0, 256, (12, 10, 3), dtype=np.uint8)
    assert np.array_equal(po.resize_linear(img, (10, 12)), img.astype(np.float32))
    assert np.array_equal(po.resize_linear(img, (10, 12), np.uint8), img)
    half = po.resize_linear(img, (5, 6))
    want = img.reshape(6, 2, 5, 2, 3).astype(np.float32).mean(axis=(1, 3))
    assert np.allclose(half, want, atol=1e-5)
    half8 = po.resize_linear(img, (5, 6), np.uint8)
    s = img.reshape(6, 2, 5, 2, 3).astype(np.int64).sum(axis=(1, 3))
    assert np.array_equal(half8, ((s + 2) >> 2).astype(np.uint8))


def test_resize_oracle_fixed_point_close_to_float():
    img = _rng().integers(0, 256, (33, 45, 3), dtype=np.uint8)
    f = po.resize_linear(img, (70, 50))
    q = po.resize_linear(img, (70, 50), np.uint8)
    # half a level of rounding plus the 11-bit weights (at most 255 / 4096 per axis)
    assert np.max(np.abs(q.astype(np.float32) - f)) <= 0.5 + 2 * 255 / 4096


# --------------------------------------------------------------------------------------------
# evaluation oracle
# --------------------------------------------------------------------------------------------
def test_psnr_closed_form():
    gt = np.full((10, 10, 3), 100, np.uint8)
    est = gt.copy()
    assert po.psnr(gt, est) == np.inf
    est[0, 0, 0] = 110
    d = np.float32(np.float32(100) / 255 - np.float32(110) / 255)
    mse = float(np.float32(d * d)) / 300
    assert po.psnr(gt, est) == pytest.approx(10 * np.log10(1 / mse), rel=1e-12)


def test_ssim_identity_and_direct_windows():
    rng = _rng(3)
    gt = rng.integers(0, 256, (12, 13, 3), dtype=np.uint8)
    assert po.ssim(gt, gt) == pytest.approx(1.0, abs=1e-12)
    est = np.clip(gt.astype(np.int32) + rng.integers(-20, 21, gt.shape), 0, 255).astype(np.uint8)
    # direct evaluation of every cropped window
    vals = []
    for ch in range(3):
        x = (gt[:, :, ch].astype(np.float32) / 255).astype(np.float64)
        y = (est[:, :, ch].astype(np.float32) / 255).astype(np.float64)
        for r in range(3, 12 - 3):
            for c in range(3, 13 - 3):
                wx, wy = x[r - 3:r + 4, c - 3:c + 4].ravel(), y[r - 3:r + 4, c - 3:c + 4].ravel()
                ux, uy = wx.mean(), wy.mean()
                vx, vy = wx.var(ddof=1), wy.var(ddof=1)
                vxy = ((wx - ux) * (wy - uy)).sum() / 48
                c1, c2 = 0.02 ** 2, 0.06 ** 2
                vals.append((2 * ux * uy + c1) * (2 * vxy + c2) / ((ux * ux + uy * uy + c1) * (vx + vy + c2)))
    assert po.ssim(gt, est) == pytest.approx(np.mean(vals), rel=1e-10)


def test_distance_errors():
    gt = np.array([[1.0, 2.0], [3.0, 4.0]], np.float32)
    est = np.array([[1.5, 2.0], [2.0, 4.25]], np.float32)
    rgb = np.zeros((2, 2, 3), np.uint8)
    # the SSIM window needs 7 x 7 images: metrics of the distances only here
    err = np.abs(est - gt)
    out = {"mae": float(err.sum() / 4), "rmse": float(np.sqrt((err * err).sum() / 4))}
    got = po.evaluate(np.zeros((8, 8, 3), np.uint8), np.pad(est, 3), np.zeros((8, 8, 3), np.uint8), np.pad(gt, 3),
                      [0.1, 0.3, 1.0])
    assert got["mae"] == pytest.approx(out["mae"] * 4 / 64)
    assert got["rmse"] == pytest.approx(np.sqrt((err * err).sum() / 64))
    assert got["bad_px_ratios"] == [100 * 3 / 64, 100 * 2 / 64, 0.0]
    assert rgb.shape == (2, 2, 3)

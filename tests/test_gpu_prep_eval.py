"""The input resize and the evaluation metrics on the GPU against their oracles
(oracle/prep_eval_oracle.py), through the C ABI: the resize bit for bit (uint8 -> float32,
float32 -> float32, uint8 -> uint8, exact 2x reductions, 1..4 channels, batches), the metrics
within float64 rounding (bad-pixel ratios exactly), and the reference-shaped helpers
read_input_images / evaluate_rgbd_panorama on files written by the package's own writers."""
from __future__ import annotations

import importlib
import os

import numpy as np
import pytest
import torch

import prep_eval_oracle as po
from conftest import PACKAGE

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def mods(native):
    return (importlib.import_module(PACKAGE + ".utils"), importlib.import_module(PACKAGE + ".evaluation"),
            importlib.import_module(PACKAGE + ".imageio"))


@pytest.mark.parametrize("src,dst,ch", [((1216, 1216), (1024, 1024), 3), ((37, 29), (64, 48), 3),
                                        ((50, 40), (31, 17), 1), ((64, 48), (32, 24), 3), ((20, 20), (20, 20), 4),
                                        ((3, 2), (9, 7), 3)])
def test_resize_matches_oracle(mods, src, dst, ch):
    utils = mods[0]
    rng = np.random.default_rng(src[0] * 7 + dst[1])
    u8 = rng.integers(0, 256, (2, src[1], src[0], ch), dtype=np.uint8)
    f32 = (rng.random((2, src[1], src[0], ch), dtype=np.float32) * 255).astype(np.float32)
    got_f = utils.resize_linear(torch.as_tensor(u8, device=DEV), dst).cpu().numpy()
    got_ff = utils.resize_linear(torch.as_tensor(f32, device=DEV), dst).cpu().numpy()
    got_q = utils.resize_linear(torch.as_tensor(u8, device=DEV), dst, out_dtype=torch.uint8).cpu().numpy()
    for i in range(2):
        assert np.array_equal(got_f[i], po.resize_linear(u8[i], dst)), "uint8 -> float32"
        assert np.array_equal(got_ff[i], po.resize_linear(f32[i], dst)), "float32 -> float32"
        assert np.array_equal(got_q[i], po.resize_linear(u8[i], dst, np.uint8)), "uint8 -> uint8"


def test_resize_rejects_bad_arguments(mods, native):
    utils = mods[0]
    with pytest.raises(ValueError):
        utils.resize_linear(torch.zeros((4, 4, 5), dtype=torch.uint8, device=DEV), (2, 2))
    with pytest.raises(ValueError):
        utils.resize_linear(torch.zeros((4, 4, 3), dtype=torch.float32, device=DEV), (2, 2), out_dtype=torch.uint8)


def _pano(rng, rows, cols):
    gt = rng.integers(0, 256, (rows, cols, 3), dtype=np.uint8)
    est = np.clip(gt.astype(np.int32) + rng.integers(-12, 13, gt.shape), 0, 255).astype(np.uint8)
    gt_inv = (rng.random((rows, cols), dtype=np.float32) * 2).astype(np.float32)
    inv = (gt_inv + rng.standard_normal((rows, cols)).astype(np.float32) * 0.05).astype(np.float32)
    return est, inv, gt, gt_inv


@pytest.mark.parametrize("rows,cols,frames", [(64, 128, 3), (7, 7, 1), (1024, 2048, 2), (33, 70, 5)])
def test_metrics_match_oracle(mods, rows, cols, frames):
    ev = mods[1]
    rng = np.random.default_rng(rows * cols)
    data = [_pano(rng, rows, cols) for _ in range(frames)]
    thr = [0.01, 0.05, 0.1]
    t = [torch.as_tensor(np.stack([d[k] for d in data]), device=DEV) for k in range(4)]
    out = ev.evaluate_panoramas(t[0], t[1], t[2], t[3], thr).cpu().numpy()
    assert out.shape == (frames, 7)
    for f, d in enumerate(data):
        want = po.evaluate(d[0], d[1], d[2], d[3], thr)
        got = ev.metrics_dict(out[f], 3)
        for k in ("psnr", "ssim", "mae", "rmse"):
            assert got[k] == pytest.approx(want[k], rel=1e-9, abs=1e-12), k
        assert got["bad_px_ratios"] == want["bad_px_ratios"]


def test_metrics_deterministic_and_identical_inputs(mods):
    ev = mods[1]
    rng = np.random.default_rng(5)
    est, inv, gt, gt_inv = _pano(rng, 256, 512)
    t = [torch.as_tensor(a, device=DEV) for a in (est, inv, gt, gt_inv)]
    a = ev.evaluate_panoramas(*t, [0.02]).cpu().numpy()
    b = ev.evaluate_panoramas(*t, [0.02]).cpu().numpy()
    assert np.array_equal(a, b)
    same = ev.evaluate_rgbd_panorama_tensors(t[2], t[3], t[2], t[3], [0.0])
    assert same["psnr"] == np.inf and same["ssim"] == pytest.approx(1.0, abs=1e-12)
    assert same["mae"] == 0.0 and same["rmse"] == 0.0 and same["bad_px_ratios"] == [0.0]


def test_metrics_reject_small_panoramas(mods):
    ev = mods[1]
    z8 = torch.zeros((6, 9, 3), dtype=torch.uint8, device=DEV)
    z32 = torch.zeros((6, 9), dtype=torch.float32, device=DEV)
    with pytest.raises(ValueError):
        ev.evaluate_panoramas(z8, z32, z8, z32)


def test_read_input_images_and_evaluate_from_files(mods, tmp_path):
    utils, ev, io = mods
    rng = np.random.default_rng(11)

    class Cal:
        original_resolution = (96, 80)

    for cam in range(3):
        os.makedirs(tmp_path / f"cam{cam}")
        io.imwrite(str(tmp_path / f"cam{cam}" / "0.png"), rng.integers(0, 256, (80, 96, 3), dtype=np.uint8))
    out = utils.read_input_images("0.png", str(tmp_path), (64, 48), (80, 60), [Cal(), Cal(), Cal()], [0, 2], DEV)
    assert out["is_valid"] and len(out["images_to_match"]) == 3 and len(out["images_to_stitch"]) == 2
    src = io.imread(str(tmp_path / "cam2" / "0.png"))
    assert np.array_equal(out["images_to_match"][2].cpu().numpy(), po.resize_linear(src, (64, 48)))
    assert np.array_equal(out["images_to_stitch"][1].cpu().numpy(), po.resize_linear(src, (80, 60)))
    with pytest.warns(UserWarning):
        bad = utils.read_input_images("1.png", str(tmp_path), (64, 48), (80, 60), [Cal()], [0], DEV)
    assert not bad["is_valid"]

    os.makedirs(tmp_path / "gt")
    est, inv, gt, gt_inv = _pano(rng, 32, 64)
    io.imwrite(str(tmp_path / "gt" / "rgb_0.png"), gt)
    io.imwrite(str(tmp_path / "gt" / "inv_distance_0.exr"), gt_inv)
    got = ev.evaluate_rgbd_panorama({"0.png": {"rgb": est, "inv_distance": inv}}, "0.png", str(tmp_path), [0.05],
                                    (64, 32), DEV)
    want = po.evaluate(est, inv, gt, gt_inv, [0.05])
    assert got["psnr"] == pytest.approx(want["psnr"], rel=1e-9)
    assert got["ssim"] == pytest.approx(want["ssim"], rel=1e-9)
    assert got["bad_px_ratios"] == want["bad_px_ratios"]
    with pytest.warns(UserWarning):
        assert ev.evaluate_rgbd_panorama({}, "0.png", str(tmp_path), [0.05], (64, 32), DEV) is None

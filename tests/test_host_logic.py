"""Host-side logic of the package, on the CPU: calibration parsing, the structs handed to the C
ABI, pyramid geometry, candidates, and the refusal of CPU devices (there is no CPU path)."""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch


def test_level_shapes_follow_the_reference(ss, oracle_mod):
    isb = __import__("importlib").import_module("sphere-stereo_gb300.isb_filter")
    o = oracle_mod.Oracle("f32")
    for cols, rows in [(1024, 1024), (768, 768), (90, 75), (33, 21), (4, 4), (5, 300)]:
        shapes = isb.level_shapes((cols, rows))
        assert len(shapes) == int(min(math.log2(cols), math.log2(rows)) - 1) == max(0, o.isb_scale_count(cols, rows))
        for s, (r, c) in enumerate(shapes):
            assert (r, c) == (math.ceil(rows / 2 ** s), math.ceil(cols / 2 ** s))


def test_level_weights():
    isb = __import__("importlib").import_module("sphere-stereo_gb300.isb_filter")
    w = isb.level_weights(9, 25.0)
    assert len(w) == 8
    for s, (up, down) in enumerate(w):
        assert down == pytest.approx(math.exp(-((2 ** s - 0.5) ** 2) / (2 * 25.0 ** 2)))
        assert up + down == pytest.approx(1.0)


def test_candidates_match_reference_formula(ss, golden_c1):
    cand = ss.distance_candidates(0.55, 100.0, 32).numpy()
    np.testing.assert_array_equal(cand, golden_c1["ref/candidates"])
    assert cand[0] == np.float32(0.55) and abs(cand[-1] - 100.0) < 1e-3


def test_calibration_structs_match_oracle(ss, oracle_mod, golden_small):
    g = golden_small
    cfg = g["config"]
    calibs = ss.parse_json_calib(g["calibration"], cfg["matching_resolution"], "cpu")
    ocams = oracle_mod.parse_calibration(g["calibration"], cfg["matching_resolution"])
    utils = __import__("importlib").import_module("sphere-stereo_gb300.utils")
    for c, oc in zip(calibs, ocams):
        k = utils.camera_struct(c)
        np.testing.assert_array_equal([k.fx, k.fy, k.cx, k.cy, k.xi, k.alpha], oracle_mod.cam6(oc))
        kk = utils.intrinsics_struct(c)
        np.testing.assert_array_equal([kk.fx, kk.fy, kk.cx, kk.cy, kk.xi, kk.alpha], oracle_mod.intrinsics_vector(oc))
    for r in cfg["references_indices"]:
        np.testing.assert_array_equal(np.array(utils.relative_poses(calibs, r), np.float32).reshape(-1, 12),
                                      oracle_mod.relative_rts(ocams, r).astype(np.float32))


def test_parse_rejects_other_camera_models(ss, golden_small):
    raw = dict(golden_small["calibration"])
    raw["intrinsics"] = [dict(i, camera_type="kb4") for i in raw["intrinsics"]]
    with pytest.raises(Exception, match="double sphere"):
        ss.parse_json_calib(raw, (64, 64), "cpu")


def test_unproject_project_round_trip(ss, golden_small):
    calibs = ss.parse_json_calib(golden_small["calibration"], (90, 75), "cpu")
    u, v = torch.meshgrid(torch.arange(10, 65, dtype=torch.float32), torch.arange(10, 80, dtype=torch.float32),
                          indexing="ij")
    uv = torch.stack([v, u], -1)
    pts, valid = ss.unproject(uv, calibs[0])
    assert valid.all()
    torch.testing.assert_close(pts.norm(dim=-1), torch.ones(pts.shape[:-1]), atol=1e-5, rtol=0)
    back, valid2 = ss.project(pts * 3.0, calibs[0])
    assert valid2.all()
    torch.testing.assert_close(back, uv, atol=2e-3, rtol=0)


def test_rgb2ycbcr_matches_oracle(ss, oracle_mod):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (20, 30, 3)).astype(np.float32)
    ours = ss.rgb2yCbCr(torch.from_numpy(img)).type(torch.uint8).numpy()
    np.testing.assert_array_equal(ours, oracle_mod.Oracle("f32").rgb2ycbcr(img))


def test_cpu_devices_are_refused(ss):
    with pytest.raises(ValueError, match="CUDA"):
        ss.ISB_Filter(4, (32, 32), "cpu")
    with pytest.raises(ValueError, match="CUDA"):
        ss.RGBD_Estimator([], 0.55, 100, 32, [0], torch.zeros(3), [], (64, 64), (64, 64), (128, 64), 10, 25, "cpu")
    with pytest.raises(ValueError, match="CUDA"):
        ss.rgb_to_guide(torch.zeros(4, 4, 3))


def test_fast_division_by_invariant_integers():
    """The multiply-high division the hole kernels use (ssg_common.cuh FastDiv), restated:
    floor(n * m / 2^(32 + s)) = floor(n / d) for every n < 2^31, m = floor(2^(32+s) / d) + 1 below
    2^32, s = floor(log2 d); powers of two shift."""
    rng = np.random.default_rng(3)
    divisors = [1, 2, 3, 5, 7, 255, 256, 1000, 1024, 1025, 1216, 1048576, 1048575, 1048577, 3 * 1048576,
                (1 << 30) + 1, (1 << 31) - 1] + [int(v) for v in rng.integers(1, 1 << 31, 200)]
    for d in divisors:
        s = d.bit_length() - 1
        m = ((1 << (32 + s)) // d + 1) if d & (d - 1) else 0
        assert m < (1 << 32)
        ns = np.concatenate([rng.integers(0, 1 << 31, 2000, dtype=np.int64),
                             np.array([0, 1, d - 1, d, d + 1, (1 << 31) - 1, (1 << 31) - d % (1 << 31)], np.int64)])
        ns = ns[(ns >= 0) & (ns < (1 << 31))].astype(object)
        for n in ns:
            q = ((n * m) >> 32) >> s if m else n >> s
            assert q == n // d, (n, d)

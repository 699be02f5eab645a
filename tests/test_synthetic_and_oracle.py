"""The synthetic workload generator and properties of the oracle itself (CPU)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import inverse_distance_mae


def test_generator_is_deterministic(synthetic):
    def frame(seed):
        rng = np.random.Generator(np.random.PCG64(seed))
        scene = synthetic.random_scene(rng)
        cams = synthetic.square_rig(96)
        return synthetic.render_frame(scene, cams, (48, 48), (64, 64), [2, 3])

    a, b, c = frame(5), frame(5), frame(6)
    for x, y in zip(a.images_to_match, b.images_to_match):
        np.testing.assert_array_equal(x, y)
    assert any((x != y).any() for x, y in zip(a.images_to_match, c.images_to_match))


def test_scene_and_rig_follow_the_spec(synthetic):
    rng = np.random.Generator(np.random.PCG64(synthetic.frame_seed(2, 3)))
    scene = synthetic.random_scene(rng)
    assert len(scene.sphere_radii) == 20
    assert np.all((scene.sphere_radii >= 0.2) & (scene.sphere_radii <= 1.0))
    assert np.all(np.linalg.norm(scene.sphere_centres, axis=1) >= scene.sphere_radii + 0.6)
    assert np.all(np.abs(scene.sphere_centres) + scene.sphere_radii[:, None] <= synthetic.ROOM_HALF + 1e-9)
    cams = synthetic.square_rig(1216)
    for k, cam in enumerate(cams):
        assert cam.fx == pytest.approx(0.28 * 1216) and cam.cx == 608
        assert np.allclose(np.abs(cam.position[[0, 2]]), 0.1) and cam.position[1] == 0
        axis = cam.rotation[:, 2]
        assert math.degrees(math.atan2(axis[0], axis[2])) % 360 == pytest.approx(45 + 90 * k)
        np.testing.assert_allclose(cam.rotation @ cam.rotation.T, np.eye(3), atol=1e-12)


def test_calibration_round_trip(synthetic, ss):
    cams = synthetic.square_rig(512)
    calibs = ss.parse_json_calib(synthetic.basalt_calibration(cams), (256, 256), "cpu")
    for c, cam in zip(calibs, cams):
        np.testing.assert_allclose(c.rt[:3, :3].numpy(), cam.rotation, atol=1e-6)
        np.testing.assert_allclose(c.rt[:3, 3].numpy(), cam.position, atol=1e-7)
        np.testing.assert_allclose(c.matching_scale.numpy(), [0.5, 0.5])


def test_ray_caster_depth_is_consistent_with_the_camera_model(synthetic):
    rng = np.random.Generator(np.random.PCG64(3))
    scene = synthetic.random_scene(rng)
    cam = synthetic.square_rig(64)[0]
    img, inv = synthetic.render_fisheye(scene, cam, 64, 64)
    valid = inv > 0
    assert valid.mean() > 0.7
    d = 1 / inv[valid]
    assert d.min() >= 0.55 - 1e-9 and d.max() <= np.linalg.norm(synthetic.ROOM_HALF) + 0.2
    assert img[~valid].max() == 0 and img[valid].std() > 10


def test_device_exponential_accuracy(oracle_mod):
    """The Cody-Waite exponential shared by the kernels and the oracle: within 2 ulp of the
    exact value over the range the filters use, 0 below the float range."""
    o = oracle_mod.Oracle("f32")
    xs = np.concatenate([np.linspace(-87, 88, 20001), -np.random.default_rng(0).random(20000) * 50,
                         [0.0, -0.0, 1e-30, -1e-30]]).astype(np.float32)
    worst = 0.0
    for x in xs:
        got = np.float32(o.cw_expf(float(x)))
        exact = math.exp(float(x))
        ulp = float(np.spacing(np.float32(exact)))
        worst = max(worst, abs(float(got) - exact) / ulp)
    assert worst <= 2.0, worst
    assert o.cw_expf(-200.0) == 0.0 and o.cw_expf(0.0) == 1.0
    assert math.isinf(o.cw_expf(100.0))
    # subnormal results are rounded once
    for x in (-90.0, -100.0, -103.0):
        assert abs(o.cw_expf(x) - math.exp(x)) <= 2 ** -149


def test_float64_oracle_agrees_with_float32(oracle_mod, golden_small):
    """The float64 restatement (the yardstick for error statements) against the float32 one.
    They are not bit-comparable: the algorithm truncates filtered guides to uint8 and takes an
    argmin, and float64 moves some of those discrete decisions.  Measured on this frame: an
    inverse-distance MAE of 1.5e-4 of the range; the bound leaves room for libm differences."""
    g = golden_small
    match = [im.astype(np.float32) for im in g["images_to_match"]]
    stitch = [im.astype(np.float32) for im in g["images_to_stitch"]]
    f32 = oracle_mod.OracleRig(g["calibration"], masks=list(g["masks"]), **g["config"]).estimate(match, stitch)
    f64 = oracle_mod.OracleRig(g["calibration"], masks=list(g["masks"]), precision="f64",
                               **g["config"]).estimate(match, stitch)
    inv_range = 1 / g["config"]["min_dist"] - 1 / g["config"]["max_dist"]
    assert inverse_distance_mae(f32["distance_filtered"], f64["distance_filtered"]) <= 1e-3 * inv_range


def test_inpaint_is_a_jacobi_step(oracle_mod):
    """One step fills a hole only from neighbours valid before the step."""
    o = oracle_mod.Oracle("f32")
    d = np.full((5, 7), 1e8, np.float32)
    d[:, 0] = 2.0
    table = np.zeros((5, 7, 2), np.uint8)
    table[..., 0] = 240 + 4 * 1 + 0   # weight 240, neighbour (dx=-1, dy=0)
    table[..., 1] = 5                 # weight 0
    one = o.inpaint(d, table, 100.0, 1)
    assert np.all(one[1:4, 1] == 2.0) and np.all(one[1:4, 2:] == 1e8)
    three = o.inpaint(d, table, 100.0, 3)
    assert np.all(three[1:4, 1:4] == 2.0) and np.all(three[1:4, 4:] == 1e8)
    assert np.all(three[0] == d[0]) and np.all(three[4] == d[4])  # borders are never filled


def test_reprojection_keeps_the_nearest(oracle_mod):
    o = oracle_mod.Oracle("f32")
    k = np.array([20, 20, 16, 16, -0.2, 0.6], np.float32)
    d = np.full((32, 32), 3.0, np.float32)
    d[10:20, 10:20] = 1.0
    out = o.reproject(d, k, np.zeros(3, np.float32))
    # zero translation: every pixel maps to itself
    np.testing.assert_allclose(out[d < 2], 1.0, rtol=1e-5)
    assert np.all(out[(d > 2) & (out < 1e8)] > 2.9)

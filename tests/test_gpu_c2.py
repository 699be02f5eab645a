"""The benchmarked configuration on the GPU: 1216^2 uint8 renders, images to match resized to
1024^2 in float32 (fractional values: the batched sweep samples them in 8.8 fixed point with 16-bit
bilinear weights), 32 candidates, sigma_s 25, references 2 and 3, stitch 1216^2, panorama
2048 x 1024.

* Against the reference's own outputs on the same inputs (tests/golden/pipeline_c2.npz, made by
  running python/depth_estimation.py:205-242 itself): the acceptance bars, for the plain fp32
  path and for the batched fp16 path the benchmark times, with the library's own rig tables
  (camera selection and relative poses computed on the GPU / host here, as in the benchmark).
* Against the oracle: the fp32 path bit for bit (distance maps, candidate indices), with the
  reference's rig tables injected so that host float32 linear algebra cannot differ.
* The stream configuration's shape (64 candidates, all four cameras as references) against the
  oracle: fp32 bit for bit, the batched fp16 path within the acceptance bars.

The inputs are regenerated from the fixture's seed and checked against its SHA-256 digests, so
they are the very bytes the reference saw; the images to match are resized by the library's GPU
resize (the benchmark's), which must reproduce the fixture's digest.
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest
import torch

from conftest import inverse_distance_mae, psnr, sample_lattice

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def c2(ss, native, synthetic, golden_c2):
    g = golden_c2
    cfg, inputs = g["config"], g["inputs"]
    w = inputs["width_in"]
    cams = synthetic.square_rig(w)
    rng = np.random.Generator(np.random.PCG64(inputs["seed"]))
    fr = synthetic.render_frame(synthetic.random_scene(rng), cams, (w, w), (w, w), [])
    renders = np.stack(fr.images_to_match)
    assert _digest(renders) == inputs["renders_sha256"], "the seeded renders differ from the reference's inputs"
    d_renders = torch.as_tensor(renders, device=DEV)
    match = ss.utils.resize_linear(d_renders, cfg["matching_resolution"])
    torch.cuda.synchronize()
    assert _digest(match.cpu().numpy()) == inputs["images_to_match_sha256"], "GPU resize differs from the fixture's"
    stitch = d_renders[cfg["references_indices"]].float().contiguous()
    assert _digest(stitch.cpu().numpy().astype(np.uint8)) == inputs["images_to_stitch_sha256"]
    return dict(g=g, cfg=cfg, renders=renders, match=match.contiguous(), stitch=stitch)


def _estimator(ss, c, storage="fp32", reference_tables=False, **override):
    g = c["g"]
    cfg = {**c["cfg"], **override}
    calibs = ss.parse_json_calib(g["calibration"], cfg["matching_resolution"], DEV)
    refs = cfg["references_indices"]
    vp = torch.zeros(3, device=DEV)
    for r in refs:
        vp += calibs[r].rt[:3, 3] / len(refs)
    cols, rows = cfg["matching_resolution"]
    masks = [torch.ones(1, rows, cols, device=DEV) for _ in calibs]
    kw = {} if storage == "fp32" else dict(cost_storage=storage, max_batch=1)
    est = ss.RGBD_Estimator(calibs, cfg["min_dist"], cfg["max_dist"], cfg["candidate_count"], refs, vp, masks,
                            cfg["matching_resolution"], cfg["rgb_to_stitch_resolution"], cfg["panorama_resolution"],
                            cfg["sigma_i"], cfg["sigma_s"], DEV, **kw)
    if reference_tables:
        est.set_rig_tables(list(g["ref/selected_cameras"]), list(g["ref/relative_poses"]))
    return est, cfg


def _bars_against_reference(label, cfg, g, index, raw, filtered, rgb, dist):
    """The acceptance bars against the reference's outputs: >= 99.9 % same candidate index (whole
    maps), inverse-distance MAE <= 1e-4 of the inverse-distance range (raw and post-filtered maps,
    panorama) and panorama RGB PSNR >= 50 dB, the last three on the fixture's 1/8 pixel lattice."""
    cols, rows = cfg["matching_resolution"]
    pw, ph = cfg["panorama_resolution"]
    stride = int(g["sample_stride"])
    pix, pano = sample_lattice(cols, rows, stride), sample_lattice(pw, ph, stride)
    R = len(cfg["references_indices"])
    inv_range = 1 / cfg["min_dist"] - 1 / cfg["max_dist"]
    same = float((index == g["ref/index"]).mean())
    mae_raw = inverse_distance_mae(raw.reshape(R, -1)[:, pix], g["ref/distance_raw@sample"]) / inv_range
    mae_f = inverse_distance_mae(filtered.reshape(R, -1)[:, pix], g["ref/distance_filtered@sample"]) / inv_range
    mae_p = inverse_distance_mae(dist.reshape(-1)[pano], g["ref/distance_panorama@sample"]) / inv_range
    p = psnr(rgb.reshape(-1, 3)[pano], g["ref/rgb_panorama@sample"])
    print(f"\n{label} vs reference: same index {same:.6f}, inverse-distance MAE / range raw {mae_raw:.2e} "
          f"filtered {mae_f:.2e} panorama {mae_p:.2e}, panorama PSNR {p:.1f} dB")
    assert same >= 0.999
    assert mae_raw <= 1e-4 and mae_f <= 1e-4 and mae_p <= 1e-4
    assert p >= 50


def test_c2_fp32_path_against_reference(ss, c2):
    est, cfg = _estimator(ss, c2)
    rgb, dist = est.estimate_RGBD_panorama(list(c2["match"]), list(c2["stitch"]))
    torch.cuda.synchronize()
    selected = torch.stack(est.selected_cameras).cpu().numpy().reshape(c2["g"]["ref/selected_cameras"].shape)
    agree = float((selected == c2["g"]["ref/selected_cameras"]).mean())
    # the reference's selection ran on the host's torch (its CPU square root is not correctly
    # rounded); near-ties between two cameras' border distances flip on ~0.01 % of the pixels
    print(f"\ncamera selection agrees with the reference's on {agree:.7f} of pixels")
    assert agree >= 0.999
    _bars_against_reference("fp32 path", cfg, c2["g"], est.index_maps.cpu().numpy(),
                            est.distance_raw_maps.cpu().numpy(), est.fishey_stitcher.distances_stacked.cpu().numpy(),
                            rgb.cpu().numpy(), dist.cpu().numpy())


@pytest.mark.parametrize("storage", ["fp16", "unorm16"])
def test_c2_batched_path_against_reference(ss, c2, storage):
    """The benchmark's path: batched, 16-bit level-0 volume, CUDA-graph replay, on the resized
    fractional inputs (every plane staged as 8.8 fixed point)."""
    est, cfg = _estimator(ss, c2, storage)
    rgb, dist = est.estimate_RGBD_panoramas(c2["match"][None].contiguous(), c2["stitch"][None].contiguous())
    torch.cuda.synchronize()
    pipe = est.pipeline()
    assert (pipe.plane_flags[:pipe.C].cpu().numpy() == 1).all(), "the resized inputs must take the 8.8 path"
    cols, rows = cfg["matching_resolution"]
    _bars_against_reference(f"batched {storage}", cfg, c2["g"], est.batch_index_maps[0].cpu().numpy(),
                            pipe.distance_raw[:2 * rows * cols].cpu().numpy(),
                            est.batch_distance_maps[0].cpu().numpy(), rgb[0].cpu().numpy(), dist[0].cpu().numpy())


def test_c2_fp32_path_bit_exact_against_oracle(ss, oracle_mod, c2):
    g = c2["g"]
    est, cfg = _estimator(ss, c2, reference_tables=True)
    rgb, dist = est.estimate_RGBD_panorama(list(c2["match"]), list(c2["stitch"]))
    torch.cuda.synchronize()
    cols, rows = cfg["matching_resolution"]
    masks = [np.ones((rows, cols), np.float32)] * 4
    rig = oracle_mod.OracleRig(g["calibration"], masks=masks, exp_mode="device", **cfg)
    rig.set_rig_tables(list(g["ref/selected_cameras"]), list(g["ref/relative_poses"]))
    ref = rig.estimate(list(c2["match"].cpu().numpy()), list(c2["stitch"].cpu().numpy()), keep_intermediates=True)
    np.testing.assert_array_equal(est.index_maps.cpu().numpy(), ref["index"])
    np.testing.assert_array_equal(est.distance_raw_maps.cpu().numpy(), ref["distance_raw"])
    np.testing.assert_array_equal(est.fishey_stitcher.distances_stacked.cpu().numpy(), ref["distance_filtered"])
    inv_range = 1 / cfg["min_dist"] - 1 / cfg["max_dist"]
    # the stitcher's sinf / cosf / norm3df are CUDA's, the oracle's libm's
    assert psnr(rgb.cpu().numpy(), ref["rgb_panorama"]) >= 50
    assert inverse_distance_mae(dist.cpu().numpy(), ref["distance_panorama"]) <= 1e-4 * inv_range


def test_c3_shape_against_oracle(ss, oracle_mod, c2):
    """64 candidates, all four cameras as references, on the same frame: the fp32 path bit for bit,
    the batched fp16 path within the acceptance bars, both against the oracle."""
    cfg = {**c2["cfg"], "candidate_count": 64, "references_indices": [0, 1, 2, 3]}
    stitch = torch.as_tensor(c2["renders"], device=DEV).float().contiguous()
    cols, rows = cfg["matching_resolution"]
    masks = [np.ones((rows, cols), np.float32)] * 4
    rig = oracle_mod.OracleRig(c2["g"]["calibration"], masks=masks, exp_mode="device", **cfg)
    ref = rig.estimate(list(c2["match"].cpu().numpy()), list(c2["renders"]), keep_intermediates=True)
    exact, _ = _estimator(ss, c2, candidate_count=64, references_indices=[0, 1, 2, 3])
    # the oracle's rig tables come from this host's float32 linear algebra; so do the library's
    exact.set_rig_tables([rig.selected[r] for r in rig.refs], [rig.rts[r] for r in rig.refs])
    rgb32, d32 = exact.estimate_RGBD_panorama(list(c2["match"]), list(stitch))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(exact.index_maps.cpu().numpy(), ref["index"])
    np.testing.assert_array_equal(exact.distance_raw_maps.cpu().numpy(), ref["distance_raw"])
    np.testing.assert_array_equal(exact.fishey_stitcher.distances_stacked.cpu().numpy(), ref["distance_filtered"])
    fast, _ = _estimator(ss, c2, "fp16", candidate_count=64, references_indices=[0, 1, 2, 3])
    fast.set_rig_tables([rig.selected[r] for r in rig.refs], [rig.rts[r] for r in rig.refs])
    rgb, dist = fast.estimate_RGBD_panoramas(c2["match"][None].contiguous(), stitch[None].contiguous())
    torch.cuda.synchronize()
    inv_range = 1 / cfg["min_dist"] - 1 / cfg["max_dist"]
    same = float((fast.batch_index_maps[0].cpu().numpy() == ref["index"]).mean())
    mae_f = inverse_distance_mae(fast.batch_distance_maps[0].cpu().numpy(), ref["distance_filtered"]) / inv_range
    mae_p = inverse_distance_mae(dist[0].cpu().numpy(), ref["distance_panorama"]) / inv_range
    p = psnr(rgb[0].cpu().numpy(), ref["rgb_panorama"])
    print(f"\n64 candidates, 4 references, batched fp16 vs oracle: same index {same:.6f}, inverse-distance "
          f"MAE / range filtered {mae_f:.2e} panorama {mae_p:.2e}, panorama PSNR {p:.1f} dB")
    assert same >= 0.999
    assert mae_f <= 1e-4 and mae_p <= 1e-4
    assert p >= 50


def test_c2_decoded_inputs_equal_the_resized_path(ss, c2):
    """The end-to-end path of the benchmark: the decoded 1216^2 uint8 renders of every camera,
    resized while they are staged, the references' renders stitched in place (no images to
    stitch).  Its outputs equal those of the resized float32 images above bit for bit, so the
    acceptance bars against the reference hold for it too."""
    est, cfg = _estimator(ss, c2, "fp16")
    rgb_f, dist_f = (t.clone() for t in est.estimate_RGBD_panoramas(c2["match"][None].contiguous(),
                                                                     c2["stitch"][None].contiguous()))
    index_f = est.batch_index_maps[0].clone()
    decoded = torch.as_tensor(c2["renders"], device=DEV)[None].contiguous()
    rgb_d, dist_d = est.estimate_RGBD_panoramas(decoded)
    torch.cuda.synchronize()
    assert torch.equal(est.batch_index_maps[0], index_f)
    assert torch.equal(rgb_d, rgb_f) and torch.equal(dist_d, dist_f)

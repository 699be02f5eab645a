"""The batched 16-bit pipeline (RGBD_Estimator(..., cost_storage="fp16" | "unorm16")) on the GPU:
acceptance bars against the reference's own outputs, batch / graph consistency, and the error
statement against the float64 oracle.

The reference's rig tables are injected (see RGBD_Estimator.set_rig_tables) so that the
comparison isolates the device path from the host's float32 linear algebra."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import inverse_distance_mae, psnr

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _estimator(ss, g, storage, max_batch=1, graphs=True, **override):
    cfg = {**g["config"], **override}
    calibs = ss.parse_json_calib(g["calibration"], cfg["matching_resolution"], DEV)
    refs = cfg["references_indices"]
    vp = torch.zeros(3, device=DEV)
    for r in refs:
        vp += calibs[r].rt[:3, 3] / len(refs)
    masks = [torch.as_tensor(m, device=DEV)[None] for m in g["masks"]]
    est = ss.RGBD_Estimator(calibs, cfg["min_dist"], cfg["max_dist"], cfg["candidate_count"], refs, vp, masks,
                            cfg["matching_resolution"], cfg["rgb_to_stitch_resolution"], cfg["panorama_resolution"],
                            cfg["sigma_i"], cfg["sigma_s"], DEV, cost_storage=storage, max_batch=max_batch,
                            cuda_graphs=graphs)
    est.set_rig_tables(list(g["ref/selected_cameras"]), list(g["ref/relative_poses"]))
    return est, cfg


def _batch(g, frames=1):
    match = torch.as_tensor(g["images_to_match"], device=DEV).float()[None].repeat(frames, 1, 1, 1, 1)
    stitch = torch.as_tensor(g["images_to_stitch"], device=DEV).float()[None].repeat(frames, 1, 1, 1, 1)
    return match.contiguous(), stitch.contiguous()


@pytest.mark.parametrize("storage", ["fp16", "unorm16"])
@pytest.mark.parametrize("name", ["small", "c1"])
def test_acceptance_against_reference(ss, native, golden_small, golden_c1, storage, name):
    g = golden_small if name == "small" else golden_c1
    est, cfg = _estimator(ss, g, storage)
    match, stitch = _batch(g)
    rgb, dist = est.estimate_RGBD_panoramas(match, stitch)
    torch.cuda.synchronize()
    inv_range = 1 / cfg["min_dist"] - 1 / cfg["max_dist"]
    index = est.batch_index_maps[0].cpu().numpy()
    same = (index == g["ref/index"]).mean()
    raw = est.pipeline().distance_raw.view(-1, *index.shape[1:])[: index.shape[0]].cpu().numpy()
    filtered = est.batch_distance_maps[0].cpu().numpy()
    mae_raw = inverse_distance_mae(raw, g["ref/distance_raw"][:, 0]) / inv_range
    mae_f = inverse_distance_mae(filtered, g["ref/distance_filtered"]) / inv_range
    mae_p = inverse_distance_mae(dist[0].cpu().numpy(), g["ref/distance_panorama"]) / inv_range
    p = psnr(rgb[0].cpu().numpy(), g["ref/rgb_panorama"])
    print(f"\n{name} {storage}: same index {same:.6f}, inverse-distance MAE / range: raw {mae_raw:.2e} "
          f"filtered {mae_f:.2e} panorama {mae_p:.2e}, panorama PSNR {p:.1f} dB")
    assert same >= 0.999
    assert mae_raw <= 1e-4 and mae_f <= 1e-4 and mae_p <= 1e-4
    assert p >= 50


def test_batch_equals_single_frames_and_graphs_equal_eager(ss, native, golden_small, synthetic):
    g = golden_small
    cfg = g["config"]
    # three different frames of the same rig
    frames = [g["images_to_match"]]
    stitches = [g["images_to_stitch"]]
    cams = synthetic.square_rig(180, 150)
    for seed in (11, 12):
        rng = np.random.Generator(np.random.PCG64(seed))
        fr = synthetic.render_frame(synthetic.random_scene(rng), cams, cfg["matching_resolution"],
                                    cfg["rgb_to_stitch_resolution"], cfg["references_indices"])
        frames.append(np.stack(fr.images_to_match))
        stitches.append(np.stack(fr.images_to_stitch))
    match = torch.as_tensor(np.stack(frames), device=DEV).float().contiguous()
    stitch = torch.as_tensor(np.stack(stitches), device=DEV).float().contiguous()
    est, _ = _estimator(ss, g, "fp16", max_batch=3, graphs=True)
    rgb3, d3 = est.estimate_RGBD_panoramas(match, stitch)
    rgb3, d3 = rgb3.clone(), d3.clone()
    eager, _ = _estimator(ss, g, "fp16", max_batch=3, graphs=False)
    rgb_e, d_e = eager.estimate_RGBD_panoramas(match, stitch)
    torch.testing.assert_close(rgb_e, rgb3, rtol=0, atol=0)
    torch.testing.assert_close(d_e, d3, rtol=0, atol=0)
    single, _ = _estimator(ss, g, "fp16", max_batch=1, graphs=True)
    for f in range(3):
        rgb1, d1 = single.estimate_RGBD_panoramas(match[f:f + 1].contiguous(), stitch[f:f + 1].contiguous())
        torch.testing.assert_close(rgb1[0], rgb3[f], rtol=0, atol=0)
        torch.testing.assert_close(d1[0], d3[f], rtol=0, atol=0)
    # replaying a cached graph after the inputs changed in place gives the new frame's result
    match2 = match.clone()
    stitch2 = stitch.clone()
    est.estimate_RGBD_panoramas(match2, stitch2)
    match2.copy_(match.flip(0))
    stitch2.copy_(stitch.flip(0))
    rgb_f, _ = est.estimate_RGBD_panoramas(match2, stitch2)
    torch.testing.assert_close(rgb_f[0], rgb3[2], rtol=0, atol=0)


def test_single_frame_api_on_16_bit_storage(ss, native, golden_small):
    g = golden_small
    est, cfg = _estimator(ss, g, "unorm16")
    match = [torch.as_tensor(im, device=DEV).float() for im in g["images_to_match"]]
    stitch = [torch.as_tensor(im, device=DEV).float() for im in g["images_to_stitch"]]
    rgb, dist = est.estimate_RGBD_panorama(match, stitch)
    torch.cuda.synchronize()
    assert rgb.shape == (64, 128, 3) and dist.shape == (64, 128)
    assert psnr(rgb.cpu().numpy(), g["ref/rgb_panorama"]) >= 50


@pytest.mark.parametrize("storage", ["fp16", "unorm16"])
def test_error_against_float64_oracle(ss, native, oracle_mod, golden_c1, storage):
    """Error statement of each output against the float64 restatement, next to the fp32 path's."""
    g = golden_c1
    est, cfg = _estimator(ss, g, storage)
    match, stitch = _batch(g)
    rgb, dist = est.estimate_RGBD_panoramas(match, stitch)
    torch.cuda.synchronize()
    rig = oracle_mod.OracleRig(g["calibration"], masks=list(g["masks"]), precision="f64", **g["config"])
    rig.set_rig_tables(list(g["ref/selected_cameras"]), list(g["ref/relative_poses"]))
    ref = rig.estimate([im.astype(np.float64) for im in g["images_to_match"]],
                       [im.astype(np.float64) for im in g["images_to_stitch"]], keep_intermediates=True)
    inv_range = 1 / cfg["min_dist"] - 1 / cfg["max_dist"]
    same = (est.batch_index_maps[0].cpu().numpy() == ref["index"]).mean()
    mae = inverse_distance_mae(est.batch_distance_maps[0].cpu().numpy(), ref["distance_filtered"]) / inv_range
    p = psnr(rgb[0].cpu().numpy(), ref["rgb_panorama"])
    f32_same = (g["ref/index"] == ref["index"]).mean()
    f32_mae = inverse_distance_mae(g["ref/distance_filtered"], ref["distance_filtered"]) / inv_range
    print(f"\nvs float64 oracle, {storage}: same index {same:.5f}, filtered inverse-distance MAE / range {mae:.2e}, "
          f"panorama PSNR {p:.1f} dB; reference fp32: same index {f32_same:.5f}, MAE / range {f32_mae:.2e}")
    # the reference's own fp32 arithmetic agrees with float64 on ~99.3 % of indices here (the
    # guide truncations and the argmin amplify rounding); the 16-bit path stays close to it
    assert same >= 0.98 and mae <= 2e-3

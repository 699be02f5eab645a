"""Rig updates without rebuilding the estimator (RGBD_Estimator.update_extrinsics): after new
camera poses or a new viewpoint, the camera selection, the stitcher's tables and every output
equal those of an estimator constructed with the new rig, on the fp32 path and on the batched
16-bit path with CUDA graphs captured before the update."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _rotation(axis, angle):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * k + (1 - np.cos(angle)) * (k @ k)


def _calibrations(ss, g, seed=None):
    cfg = g["config"]
    calibs = ss.parse_json_calib(g["calibration"], cfg["matching_resolution"], DEV)
    if seed is not None:
        rng = np.random.default_rng(seed)
        for c in calibs:
            rt = c.rt.double().cpu().numpy()
            rp = _rotation(rng.standard_normal(3), np.deg2rad(0.5))
            out = np.eye(4)
            out[:3, :3] = rp @ rt[:3, :3]
            out[:3, 3] = rp @ rt[:3, 3] + rng.standard_normal(3) * 0.005
            c.rt = torch.as_tensor(out, dtype=torch.float32, device=DEV)
    return calibs


def _viewpoint(calibs, refs):
    vp = torch.zeros(3, device=DEV)
    for r in refs:
        vp += calibs[r].rt[:3, 3] / len(refs)
    return vp


def _estimator(ss, g, calibs, vp, storage, graphs=True):
    cfg = g["config"]
    masks = [torch.as_tensor(m, device=DEV)[None] for m in g["masks"]]
    return ss.RGBD_Estimator(calibs, cfg["min_dist"], cfg["max_dist"], cfg["candidate_count"],
                             cfg["references_indices"], vp, masks, cfg["matching_resolution"],
                             cfg["rgb_to_stitch_resolution"], cfg["panorama_resolution"], cfg["sigma_i"],
                             cfg["sigma_s"], DEV, cost_storage=storage, max_batch=2, cuda_graphs=graphs)


def _same_rig(a, b):
    for x, y in zip(a.selected_cameras, b.selected_cameras):
        assert torch.equal(x, y)
    sa, sb = a.fishey_stitcher, b.fishey_stitcher
    assert torch.equal(sa.translations, sb.translations)
    assert torch.equal(sa.blending_sampling, sb.blending_sampling)
    assert torch.equal(sa.blending_weights, sb.blending_weights)
    for x, y in zip(sa.inpainting_weights_list, sb.inpainting_weights_list):
        assert torch.equal(x, y)


def _frames(g):
    match = torch.as_tensor(g["images_to_match"], device=DEV).float()
    stitch = torch.as_tensor(g["images_to_stitch"], device=DEV).float()
    return match, stitch


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_update_extrinsics_equals_a_new_estimator(ss, native, golden_small, storage):
    g = golden_small
    refs = g["config"]["references_indices"]
    old = _calibrations(ss, g)
    new = _calibrations(ss, g, seed=5)
    est = _estimator(ss, g, old, _viewpoint(old, refs), storage)
    fresh = _estimator(ss, g, new, _viewpoint(old, refs), storage)
    match, stitch = _frames(g)
    batch = (torch.stack([match, match.flip(0)]).contiguous(), torch.stack([stitch, stitch]).contiguous())

    def run(e):
        if storage == "fp32":
            rgb, d = e.estimate_RGBD_panorama(list(match), list(stitch))
            return rgb.clone(), d.clone()
        rgb, d = e.estimate_RGBD_panoramas(*batch)
        return rgb.clone(), d.clone()

    before = run(est)  # a graph is captured with the old rig
    est.update_extrinsics([c.rt for c in new])
    _same_rig(est, fresh)
    after, want = run(est), run(fresh)
    assert not torch.equal(before[1], after[1])
    torch.testing.assert_close(after[0], want[0], rtol=0, atol=0)
    torch.testing.assert_close(after[1], want[1], rtol=0, atol=0)

    # a new viewpoint alone
    vp2 = _viewpoint(new, refs) + torch.tensor([0.01, -0.02, 0.015], device=DEV)
    est.update_extrinsics(reprojection_viewpoint=vp2)
    moved = _estimator(ss, g, _calibrations(ss, g, seed=5), vp2, storage)
    _same_rig(est, moved)
    got, want = run(est), run(moved)
    torch.testing.assert_close(got[0], want[0], rtol=0, atol=0)
    torch.testing.assert_close(got[1], want[1], rtol=0, atol=0)


def test_update_extrinsics_rejects_bad_poses(ss, native, golden_small):
    g = golden_small
    calibs = _calibrations(ss, g)
    est = _estimator(ss, g, calibs, _viewpoint(calibs, g["config"]["references_indices"]), "fp16")
    with pytest.raises(ValueError):
        est.update_extrinsics([torch.eye(4)] * (len(calibs) - 1))
    with pytest.raises(ValueError):
        est.update_extrinsics([torch.full((4, 4), float("nan"))] * len(calibs))

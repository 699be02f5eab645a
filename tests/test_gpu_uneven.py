"""Uneven batches (UnevenBatch / ssg_uneven_*): jobs of different rigs, matching resolutions and
candidate counts in one launch sequence.  Every job must give exactly what the uniform batched
path gives for that rig alone: the persistent sweep, the descriptor-driven filter steps and the
stitch over concatenated maps run the same per-pixel arithmetic."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"

# (matching width, candidates, cameras, references) per job; rigs and scenes are seeded per job
JOBS = [(128, 16, 3, [0, 1]), (192, 24, 5, [1, 3]), (160, 40, 4, [2]), (128, 8, 6, [0, 2, 4])]


def _job(ss, synthetic, k, width, candidates, cameras, refs):
    rng = np.random.Generator(np.random.PCG64(synthetic.frame_seed(5, k)))
    cams = synthetic.ring_rig(rng, width, cameras)
    scene = synthetic.random_scene(rng)
    frame = synthetic.render_frame(scene, cams, (width, width), (width, width), refs)
    calibs = ss.parse_json_calib(synthetic.basalt_calibration(cams), (width, width), DEV)
    vp = torch.zeros(3, device=DEV)
    for r in refs:
        vp += calibs[r].rt[:3, 3] / len(refs)
    masks = [torch.ones(1, width, width, device=DEV) for _ in cams]
    est = ss.RGBD_Estimator(calibs, 0.55, 100.0, candidates, refs, vp, masks, (width, width), (width, width),
                            (2 * width, width), 10.0, 6.25, DEV, cost_storage="fp16", max_batch=1)
    match = torch.as_tensor(np.stack(frame.images_to_match), device=DEV).float().contiguous()
    stitch = torch.as_tensor(np.stack(frame.images_to_stitch), device=DEV).float().contiguous()
    return est, match, stitch


@pytest.fixture(scope="module")
def jobs(ss, native, synthetic):
    return [_job(ss, synthetic, k, *spec) for k, spec in enumerate(JOBS)]


@pytest.mark.parametrize("graphs", [False, True])
def test_uneven_batch_equals_each_rig_alone(ss, jobs, graphs):
    from importlib import import_module

    uneven = import_module("sphere-stereo_gb300.uneven")
    batch = uneven.UnevenBatch([e for e, _, _ in jobs], cuda_graphs=graphs)
    for _ in range(2):  # a second run (graph replay) gives the same outputs
        outs = batch.run([m for _, m, _ in jobs], [s for _, _, s in jobs])
        torch.cuda.synchronize()
        idx_u = [t.cpu().numpy() for t in batch.index_maps]
        dist_u = [t.cpu().numpy() for t in batch.distance_maps]
        raw_u = [t.cpu().numpy() for t in batch.raw_distance_maps]
        pano_u = [(r.cpu().numpy(), d.cpu().numpy()) for r, d in outs]
        for k, (est, match, stitch) in enumerate(jobs):
            rgb, dist = est.estimate_RGBD_panoramas(match[None].contiguous(), stitch[None].contiguous())
            torch.cuda.synchronize()
            p = est.pipeline()
            R = len(est.references_indices)
            np.testing.assert_array_equal(idx_u[k], est.batch_index_maps[0].cpu().numpy(), err_msg=f"job {k} index")
            np.testing.assert_array_equal(raw_u[k], p.distance_raw.view(-1, R, *idx_u[k].shape[1:])[0].cpu().numpy(),
                                          err_msg=f"job {k} raw distance")
            np.testing.assert_array_equal(dist_u[k], est.batch_distance_maps[0].cpu().numpy(),
                                          err_msg=f"job {k} distance")
            np.testing.assert_array_equal(pano_u[k][0], rgb[0].cpu().numpy(), err_msg=f"job {k} rgb")
            np.testing.assert_array_equal(pano_u[k][1], dist[0].cpu().numpy(), err_msg=f"job {k} panorama")


def test_uneven_batch_uint8_inputs(ss, jobs):
    from importlib import import_module

    uneven = import_module("sphere-stereo_gb300.uneven")
    f32 = uneven.UnevenBatch([e for e, _, _ in jobs], cuda_graphs=False)
    u8 = uneven.UnevenBatch([e for e, _, _ in jobs], cuda_graphs=True, input_dtype=torch.uint8)
    a = f32.run([m for _, m, _ in jobs], [s for _, _, s in jobs])
    b = u8.run([m.to(torch.uint8) for _, m, _ in jobs], [s.to(torch.uint8) for _, _, s in jobs])
    torch.cuda.synchronize()
    for (ra, da), (rb, db) in zip(a, b):
        assert torch.equal(ra, rb) and torch.equal(da, db)
    assert u8.launches() == f32.launches() - len(jobs)  # no float -> uint8 conversion per job


def test_uneven_rejects_invalid_jobs(ss, jobs):
    from importlib import import_module

    uneven = import_module("sphere-stereo_gb300.uneven")
    with pytest.raises(ValueError):
        uneven.UnevenBatch([])
    with pytest.raises(ValueError):
        uneven.UnevenBatch([jobs[0][0]], storage="fp8")

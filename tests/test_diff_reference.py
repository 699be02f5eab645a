"""The float64 autograd restatement of the differentiable sweep (oracle/diff_reference.py), the
yardstick of the CUDA backward, against central finite differences on the CPU.

The cost is piecewise linear in the pose (L1 of bilinear samples, clamped), so pose
differences converge to the derivative only for steps small enough to cross no kink; a step of
1e-7 in float64 does, a step of 1e-4 differs by a few percent.  The image gradient is checked at
the step of 1e-4."""
from __future__ import annotations

import numpy as np
import pytest
import torch


@pytest.fixture(scope="module")
def tiny(synthetic, oracle_mod):
    import diff_reference

    res = (40, 40)
    cams = synthetic.square_rig(80)
    rng = np.random.Generator(np.random.PCG64(synthetic.frame_seed(4, 1)))
    frame = synthetic.render_frame(synthetic.random_scene(rng), cams, res, res, [2, 3])
    noisy = synthetic.perturb_rig(cams, np.random.Generator(np.random.PCG64(4001)), 0.5, 0.005)
    calibration = synthetic.basalt_calibration(noisy)
    kw = dict(min_dist=0.55, max_dist=100.0, candidate_count=8, references_indices=[2, 3], sigma_i=10.0, sigma_s=6.25)
    rig = oracle_mod.OracleRig(calibration, masks=[np.ones((40, 40))] * 4, matching_resolution=res,
                               rgb_to_stitch_resolution=res, panorama_resolution=(32, 16), exp_mode="device", **kw)
    images = np.stack(frame.images_to_match).astype(np.float64)
    guides = [rig.o.rgb2ycbcr(images[r].astype(np.float32)) for r in kw["references_indices"]]
    ref = diff_reference.DiffReference(calibration, matching_resolution=res,
                                       selected=[rig.selected[r] for r in kw["references_indices"]], guides=guides,
                                       temperature=2.0, **kw)
    gt = torch.as_tensor(np.stack([frame.inv_distance[r] for r in kw["references_indices"]]))
    return ref, torch.as_tensor(images), gt


def _loss(q, gt):
    valid = gt > 0
    return (q - gt).abs()[valid].mean()


def test_autograd_matches_central_differences(tiny):
    ref, images, gt = tiny
    im = images.clone().requires_grad_()
    de = torch.zeros(4, 6, dtype=torch.float64, requires_grad=True)
    _loss(ref.inverse_distance(im, de), gt).backward()

    def f(im_, de_):
        with torch.no_grad():
            return _loss(ref.inverse_distance(im_, de_), gt).item()

    zero = torch.zeros(4, 6, dtype=torch.float64)
    fd = torch.zeros(4, 6, dtype=torch.float64)
    h = 1e-7
    for c in range(4):
        for j in range(6):
            e = zero.clone()
            e[c, j] = h
            fd[c, j] = (f(images, e) - f(images, -e)) / (2 * h)
    assert ((de.grad - fd).norm() / fd.norm()).item() <= 1e-3
    rng = np.random.default_rng(0)
    nz = torch.nonzero(im.grad.abs() > 1e-8)
    num, ana = [], []
    for i in rng.choice(len(nz), 12, replace=False):
        c, y, x, ch = nz[i].tolist()
        e = torch.zeros_like(images)
        e[c, y, x, ch] = 1e-4
        num.append((f(images + e, zero) - f(images - e, zero)) / 2e-4)
        ana.append(im.grad[c, y, x, ch].item())
    num, ana = np.array(num), np.array(ana)
    assert np.linalg.norm(num - ana) / np.linalg.norm(num) <= 1e-3


def test_zero_delta_is_the_calibrated_rig(tiny):
    ref, images, _ = tiny
    q0 = ref.inverse_distance(images, torch.zeros(4, 6, dtype=torch.float64))
    assert torch.isfinite(q0).all()
    c = ref.cand
    assert (q0 >= 1 / c.max() - 1e-12).all() and (q0 <= 1 / c.min() + 1e-12).all()

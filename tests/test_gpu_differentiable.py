"""The differentiable sweep (soft-argmin inverse distance, gradients with respect to the images
and to each camera's 6-DoF pose delta) against a float64 torch autograd restatement
(oracle/diff_reference.py) and central finite differences.

Setting, after the differentiable-sweep configuration at reduced size: the synthetic rig's
extrinsics perturbed by a seeded 0.5 deg rotation and 5 mm translation, images ray-cast with
the true rig, loss = L1 between the soft-argmin inverse distance and the ray-cast ground truth.

The cost is an L1 of bilinear samples with a clamp: piecewise linear in the pose, so a central
difference with a pose step of 1e-4 rad / 1e-4 m crosses many of its kinks and differs from the
derivative by a few percent; with a step of 1e-7 the differences converge to the derivative.
Image steps of 1e-4 (intensity units) cross almost none.
"""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def setting(ss, native, synthetic, oracle_mod):
    import diff_reference

    res = (96, 96)
    true_cams = synthetic.square_rig(192)
    rng = np.random.Generator(np.random.PCG64(synthetic.frame_seed(4, 0)))
    scene = synthetic.random_scene(rng)
    frame = synthetic.render_frame(scene, true_cams, res, res, [2, 3])
    noisy = synthetic.perturb_rig(true_cams, np.random.Generator(np.random.PCG64(4000)), 0.5, 0.005)
    calibration = synthetic.basalt_calibration(noisy)
    calibs = ss.parse_json_calib(calibration, res, DEV)
    masks = [torch.ones(1, res[1], res[0], device=DEV) for _ in calibs]
    kw = dict(min_dist=0.55, max_dist=100.0, candidate_count=16, references_indices=[2, 3], sigma_i=10.0,
              sigma_s=6.25)
    sweep = ss.DifferentiableSweep(calibs, kw["min_dist"], kw["max_dist"], kw["candidate_count"],
                                   kw["references_indices"], masks, res, kw["sigma_i"], kw["sigma_s"], DEV,
                                   temperature=2.0)
    images = np.stack(frame.images_to_match).astype(np.float32)
    gt = np.stack([frame.inv_distance[r] for r in kw["references_indices"]])
    guides = [oracle_mod.Oracle("f32", exp_mode="device").rgb2ycbcr(images[r]) for r in kw["references_indices"]]
    ref = diff_reference.DiffReference(calibration, matching_resolution=res, selected=[s.cpu().numpy()
                                                                                       for s in sweep.selected],
                                       guides=guides, temperature=2.0, **kw)
    return sweep, ref, images, gt


def _loss(q, gt):
    valid = gt > 0
    return (q - gt).abs()[valid].mean()


def test_forward_matches_float64(setting):
    """fp32 evaluation of the float64 formula: the relative poses are rounded to float32, which
    moves samples by ~1e-5 px and costs (magnitude ~100) by ~1e-3; through softmax(-F / 2) that
    is a relative weight change of ~5e-4 on an inverse distance range of 1.8, so the bound is
    3e-5 absolute (1.7e-5 of the range)."""
    sweep, ref, images, gt = setting
    q = sweep(torch.as_tensor(images, device=DEV)).cpu().double()
    q64 = ref.inverse_distance(torch.as_tensor(images, dtype=torch.float64), torch.zeros(4, 6, dtype=torch.float64))
    err = (q - q64).abs().max().item()
    print(f"\nsoft-argmin inverse distance vs float64: max abs error {err:.2e}")
    assert err <= 3e-5


def test_gradients_are_bit_reproducible(setting):
    """Two backward passes of the same inputs give the same bits: the transposed filter steps
    gather in a fixed order, the image gradient is summed in 64-bit fixed point, and the pose
    gradient by a fixed float64 tree (no float atomic adds)."""
    sweep, ref, images, gt = setting
    gt_t = torch.as_tensor(gt)
    grads = []
    for _ in range(3):
        im = torch.as_tensor(images, device=DEV).requires_grad_()
        de = torch.zeros(4, 6, dtype=torch.float64, device=DEV, requires_grad=True)
        _loss(sweep(im, de).double().cpu(), gt_t).backward()
        grads.append((im.grad.cpu().numpy(), de.grad.cpu().numpy()))
    assert np.abs(grads[0][0]).max() > 0 and np.abs(grads[0][1]).max() > 0
    for g_im, g_de in grads[1:]:
        np.testing.assert_array_equal(g_im, grads[0][0])
        np.testing.assert_array_equal(g_de, grads[0][1])


def test_gradients_match_float64_autograd_and_finite_differences(setting):
    sweep, ref, images, gt = setting
    gt_t = torch.as_tensor(gt)
    im = torch.as_tensor(images, device=DEV).requires_grad_()
    de = torch.zeros(4, 6, dtype=torch.float64, device=DEV, requires_grad=True)
    loss = _loss(sweep(im, de).double().cpu(), gt_t)
    loss.backward()
    g_im, g_de = im.grad.double().cpu(), de.grad.cpu()

    im64 = torch.as_tensor(images, dtype=torch.float64).requires_grad_()
    de64 = torch.zeros(4, 6, dtype=torch.float64, requires_grad=True)
    loss64 = _loss(ref.inverse_distance(im64, de64), gt_t)
    loss64.backward()
    r_pose = ((g_de - de64.grad).norm() / de64.grad.norm()).item()
    r_img = ((g_im - im64.grad).norm() / im64.grad.norm()).item()

    def f64(im_, de_):
        with torch.no_grad():
            return _loss(ref.inverse_distance(im_, de_), gt_t).item()

    base_im = im64.detach()
    zero = torch.zeros(4, 6, dtype=torch.float64)
    fd = {}
    for h in (1e-4, 1e-7):
        d = torch.zeros(4, 6, dtype=torch.float64)
        for c in range(4):
            for j in range(6):
                e = zero.clone()
                e[c, j] = h
                d[c, j] = (f64(base_im, e) - f64(base_im, -e)) / (2 * h)
        fd[h] = ((g_de - d).norm() / d.norm()).item()
    rng = np.random.default_rng(1)
    nz = torch.nonzero(im64.grad.abs() > 1e-8)
    picks = [tuple(nz[i].tolist()) for i in rng.choice(len(nz), 96, replace=False)]
    fd_img, ana = [], []
    for (c, y, x, ch) in picks:
        e = torch.zeros_like(base_im)
        e[c, y, x, ch] = 1e-4
        fd_img.append((f64(base_im + e, zero) - f64(base_im - e, zero)) / 2e-4)
        ana.append(g_im[c, y, x, ch].item())
    fd_img, ana = np.array(fd_img), np.array(ana)
    r_fd_img = float(np.linalg.norm(fd_img - ana) / np.linalg.norm(fd_img))
    # control: the float64 reference's own gradient against the same central differences
    d = torch.zeros(4, 6, dtype=torch.float64)
    for c in range(4):
        for j in range(6):
            e = zero.clone()
            e[c, j] = 1e-4
            d[c, j] = (f64(base_im, e) - f64(base_im, -e)) / 2e-4
    fd_ref = ((de64.grad - d).norm() / d.norm()).item()
    print(f"\nrelative error vs float64 autograd: poses {r_pose:.2e}, images {r_img:.2e}; vs central differences: "
          f"poses (step 1e-4) {fd[1e-4]:.2e} (float64 autograd at the same step: {fd_ref:.2e}), "
          f"poses (step 1e-7) {fd[1e-7]:.2e}, images (step 1e-4) {r_fd_img:.2e}")
    assert r_pose <= 1e-3 and r_img <= 1e-3
    assert fd[1e-7] <= 1e-3
    assert r_fd_img <= 1e-3
    # at step 1e-4 the difference quotient crosses kinks of the L1 cost: the bar is 1e-3, or, where
    # the exact float64 gradient itself misses it, that gradient's own error at the same step
    assert math.isfinite(fd[1e-4])
    assert fd[1e-4] <= 1e-3 or fd[1e-4] <= 1.05 * fd_ref + 1e-3


def test_descent_on_pose_deltas_reduces_the_loss(setting):
    """A few gradient steps on the pose deltas (calibration refinement) lower the loss."""
    sweep, _, images, gt = setting
    gt_t = torch.as_tensor(gt)
    im = torch.as_tensor(images, device=DEV)
    de = torch.zeros(4, 6, dtype=torch.float64, device=DEV, requires_grad=True)
    opt = torch.optim.Adam([de], lr=2e-3)
    losses = []
    for _ in range(8):
        opt.zero_grad()
        loss = _loss(sweep(im, de).double().cpu(), gt_t)
        loss.backward()
        opt.step()
        losses.append(loss.item())
    print("\nloss during refinement:", " ".join(f"{v:.4f}" for v in losses))
    assert losses[-1] < losses[0]


# ---------------------------------------------------------------------------------------------
# The differentiable-sweep configuration at full size: 8 frames at 512 x 512 matching, 48
# candidates, the rig's extrinsics perturbed by a seeded 0.5 deg rotation and 5 mm translation,
# images ray-cast with the true rig, loss = mean over frames of the L1 between the soft-argmin
# inverse distance and the ray-cast ground truth.  The float64 reference runs on the GPU.
# ---------------------------------------------------------------------------------------------
C4 = dict(res=(512, 512), frames=8, min_dist=0.55, max_dist=100.0, candidate_count=48, references_indices=[2, 3],
          sigma_i=10.0, sigma_s=25.0, temperature=2.0)


@pytest.fixture(scope="module")
def c4(ss, native, synthetic, oracle_mod):
    import diff_reference

    res = C4["res"]
    true_cams = synthetic.square_rig(res[0])
    noisy = synthetic.perturb_rig(true_cams, np.random.Generator(np.random.PCG64(4000)), 0.5, 0.005)
    calibration = synthetic.basalt_calibration(noisy)
    calibs = ss.parse_json_calib(calibration, res, DEV)
    masks = [torch.ones(1, res[1], res[0], device=DEV) for _ in calibs]
    kw = {k: C4[k] for k in ("min_dist", "max_dist", "candidate_count", "references_indices", "sigma_i", "sigma_s")}
    sweep = ss.DifferentiableSweep(calibs, kw["min_dist"], kw["max_dist"], kw["candidate_count"],
                                   kw["references_indices"], masks, res, kw["sigma_i"], kw["sigma_s"], DEV,
                                   temperature=C4["temperature"])
    selected = [s.cpu().numpy() for s in sweep.selected]
    o = oracle_mod.Oracle("f32", exp_mode="device")
    frames = []
    for f in range(C4["frames"]):
        rng = np.random.Generator(np.random.PCG64(synthetic.frame_seed(4, f)))
        fr = synthetic.render_frame(synthetic.random_scene(rng), true_cams, res, res, [])
        images = np.stack(fr.images_to_match).astype(np.float32)
        gt = torch.as_tensor(np.stack([fr.inv_distance[r] for r in kw["references_indices"]]), device=DEV)
        ref = diff_reference.DiffReference(calibration, matching_resolution=res, selected=selected,
                                           guides=[o.rgb2ycbcr(images[r]) for r in kw["references_indices"]],
                                           temperature=C4["temperature"], device=DEV, **kw)
        frames.append((images, gt, ref))
    return sweep, frames


def _c4_loss64(frames, deltas):
    total = 0.0
    for im, gt, ref in frames:
        total = total + _loss(ref.inverse_distance(torch.as_tensor(im, dtype=torch.float64, device=DEV), deltas), gt)
    return total / len(frames)


def test_c4_gradients_at_full_size(c4):
    """Gradients of the 8-frame loss with respect to the 6-DoF pose deltas and the images: the same
    bits from a second backward; against central differences of the float64 loss (relative error
    <= 1e-3 at step 1e-4, with the float64 gradient's own error at that step as the control, and at
    step 1e-7) and against float64 autograd (bars below)."""
    sweep, frames = c4
    de = torch.zeros(4, 6, dtype=torch.float64, device=DEV, requires_grad=True)
    ims = [torch.as_tensor(im, device=DEV).requires_grad_() for im, _, _ in frames]
    loss = sum(_loss(sweep(x, de).double(), gt) for x, (_, gt, _) in zip(ims, frames)) / len(frames)
    loss.backward()
    g_de = de.grad.detach().cpu()
    g_im = [x.grad.detach().double() for x in ims]
    # a second backward of the same inputs gives the same bits
    de2 = torch.zeros(4, 6, dtype=torch.float64, device=DEV, requires_grad=True)
    ims2 = [torch.as_tensor(im, device=DEV).requires_grad_() for im, _, _ in frames]
    (sum(_loss(sweep(x, de2).double(), gt) for x, (_, gt, _) in zip(ims2, frames)) / len(frames)).backward()
    assert torch.equal(de2.grad.cpu(), g_de)
    assert all(torch.equal(a.grad, b.grad) for a, b in zip(ims2, ims))

    # float64 autograd one frame at a time (each frame's graph holds ~20 GB of intermediates)
    de64 = torch.zeros(4, 6, dtype=torch.float64, device=DEV, requires_grad=True)
    ims64 = [torch.as_tensor(im, dtype=torch.float64, device=DEV).requires_grad_() for im, _, _ in frames]
    loss64 = 0.0
    for x, (_, gt, ref) in zip(ims64, frames):
        lf = _loss(ref.inverse_distance(x, de64), gt) / len(frames)
        lf.backward()
        loss64 += lf.item()
    g64_de = de64.grad.detach().cpu()
    r_pose = ((g_de - g64_de).norm() / g64_de.norm()).item()
    r_img = (torch.sqrt(sum(((a - x.grad) ** 2).sum() for a, x in zip(g_im, ims64))) /
             torch.sqrt(sum((x.grad ** 2).sum() for x in ims64))).item()
    print(f"\nloss: device {loss.item():.6f}, float64 {loss64:.6f}")

    def fd_pose(h):
        d = torch.zeros(4, 6, dtype=torch.float64)
        with torch.no_grad():
            for c in range(4):
                for j in range(6):
                    e = torch.zeros(4, 6, dtype=torch.float64, device=DEV)
                    e[c, j] = h
                    d[c, j] = (_c4_loss64(frames, e) - _c4_loss64(frames, -e)).item() / (2 * h)
        return d

    fd4, fd7 = fd_pose(1e-4), fd_pose(1e-7)
    e4 = ((g_de - fd4).norm() / fd4.norm()).item()
    e4_ref = ((g64_de - fd4).norm() / fd4.norm()).item()
    e7 = ((g_de - fd7).norm() / fd7.norm()).item()
    # image entries: central differences (step 1e-4) of the float64 loss at 64 seeded texels of
    # two frames (a texel only moves its own frame's term)
    rng = np.random.default_rng(4)
    zero = torch.zeros(4, 6, dtype=torch.float64, device=DEV)
    fd_img, ana = [], []
    with torch.no_grad():
        for f in (0, 5):
            im, gt, ref = frames[f]
            base = torch.as_tensor(im, dtype=torch.float64, device=DEV)
            nz = torch.nonzero(ims64[f].grad.abs() > 1e-9)
            for i in rng.choice(len(nz), 32, replace=False):
                c, y, x, ch = nz[i].tolist()
                e = torch.zeros_like(base)
                e[c, y, x, ch] = 1e-4
                plus = _loss(ref.inverse_distance(base + e, zero), gt).item()
                minus = _loss(ref.inverse_distance(base - e, zero), gt).item()
                fd_img.append((plus - minus) / 2e-4 / len(frames))
                ana.append(g_im[f][c, y, x, ch].item())
    fd_img, ana = np.array(fd_img), np.array(ana)
    r_fd_img = float(np.linalg.norm(fd_img - ana) / np.linalg.norm(fd_img))
    print(f"8 frames, 512^2, 48 candidates: relative error vs float64 autograd: poses {r_pose:.2e}, images "
          f"{r_img:.2e}; vs central differences: poses (step 1e-4) {e4:.2e} (float64 autograd at the same step: "
          f"{e4_ref:.2e}), poses (step 1e-7) {e7:.2e}, images (step 1e-4) {r_fd_img:.2e}")
    # the finite-difference checks hold at 1e-3.  Against float64 autograd the image gradient
    # differs by ~1.5e-3 at this size: the device evaluates the forward in float32 (samples move by
    # ~1e-5 px, costs by ~1e-3, and L1 residuals within that of zero take the other side of the
    # kink), and the image gradient, a scatter of those per-sample signs, carries it; the bar for
    # that comparison is 2e-3
    assert r_pose <= 1e-3 and r_img <= 2e-3
    assert e7 <= 1e-3
    assert r_fd_img <= 1e-3
    assert e4 <= 1e-3 or e4 <= 1.05 * e4_ref + 1e-3

"""Resize and staging in one pass (ssg_stage_images_resized): the decoded 8-bit images of every
camera, resized to the matching resolution while they are staged, must give exactly what the
two passes give -- ssg_resize_linear (u8 -> float32, the reference's input preparation,
python/utils.py:198-201) followed by ssg_stage_images -- entries, guides and plane flags bit for
bit; and the batched pipeline fed the decoded images must give the outputs it gives for the
resized float32 images."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _stage_both(N, imgs: np.ndarray, cols: int, rows: int, refs: list[int], columns: int):
    """imgs: uint8 [frames, cameras, H, W, 3].  Returns ((staged, guides, flags) two-pass with the
    shared-memory tile staging, (staged, guides, flags) one-pass with the staging kernel
    `columns` selects) as numpy arrays."""
    F, C, H, W, _ = imgs.shape
    src = torch.as_tensor(imgs, device=DEV)
    stream = torch.cuda.current_stream().cuda_stream
    plane = (rows + 2) * (cols + 2)
    out = []
    for fused in (False, True):
        N.call("ssg_tuning_set", N.TUNE_STAGE_COLUMNS, columns if fused else 0)
        staged = torch.full((F * C * 2 * plane * 4,), 7.0, device=DEV)  # a pattern every entry overwrites
        guides = torch.zeros(F * len(refs) * rows * cols * 4, dtype=torch.uint8, device=DEV)
        flags = torch.full((F * C,), -1, dtype=torch.int32, device=DEV)
        if fused:
            N.call("ssg_stage_images_resized", src.data_ptr(), W, H, F, C, cols, rows, N.ints(refs), len(refs),
                   staged.data_ptr(), guides.data_ptr(), flags.data_ptr(), stream)
        else:
            resized = torch.empty((F * C, rows, cols, 3), dtype=torch.float32, device=DEV)
            N.call("ssg_resize_linear", src.data_ptr(), N.PIXEL_U8, W, H, 3, resized.data_ptr(), N.PIXEL_F32, cols,
                   rows, F * C, stream)
            N.call("ssg_stage_images", resized.data_ptr(), F, C, cols, rows, N.ints(refs), len(refs),
                   staged.data_ptr(), guides.data_ptr(), flags.data_ptr(), stream)
        torch.cuda.synchronize()
        out.append((staged.cpu().numpy().view(np.uint32), guides.cpu().numpy(), flags.cpu().numpy()))
    return out


# (source W, H) -> (matching cols, rows): the benchmark's 1216^2 -> 1024^2, an exact 2x reduction
# (area average), enlargements, uneven factors, and a reduction whose tile windows need more
# than 48 KB of shared memory
CASES = [((1216, 1216), (1024, 1024)), ((200, 120), (100, 60)), ((100, 60), (130, 70)), ((96, 75), (90, 75)),
         ((64, 36), (150, 101)), ((1216, 1216), (512, 512)), ((333, 212), (257, 161))]


@pytest.mark.parametrize("columns", [1, 0])
@pytest.mark.parametrize("src,dst", CASES)
def test_stage_resized_equals_resize_then_stage(ss, native, src, dst, columns):
    """Both staging kernels (SSG_TUNE_STAGE_COLUMNS: warps walking down column strips, or
    shared-memory texel tiles) against the two passes."""
    N = ss._native
    rng = np.random.default_rng(sum(src) + 7 * sum(dst))
    (W, H), (cols, rows) = src, dst
    frames, cams = (1, 4) if W * H > 10 ** 6 else (2, 3)
    imgs = rng.integers(0, 256, (frames, cams, H, W, 3), dtype=np.uint8)
    imgs[0, 0, : H // 3] = 255  # saturated and flat regions next to noise
    imgs[-1, -1, :, : W // 4] = 0
    (s2, g2, f2), (s1, g1, f1) = _stage_both(N, imgs, cols, rows, [0, cams - 1], columns)
    np.testing.assert_array_equal(f1, f2)
    np.testing.assert_array_equal(g1, g2)
    np.testing.assert_array_equal(s1, s2)
    assert set(f1.tolist()) <= {0, 1}  # resized 8-bit values never take the float path


def test_stage_resized_declines_unaligned_sources(ss, native):
    """A source whose images do not start on 4-byte boundaries is declined before any launch with
    SSG_ERR_UNSUPPORTED (the caller resizes first); nothing is written."""
    N = ss._native
    src = torch.zeros(1 * 2 * 35 * 33 * 3, dtype=torch.uint8, device=DEV)  # 35 x 33 pixels: 1155, odd
    staged = torch.zeros(2 * 2 * 22 * 22 * 4, device=DEV)
    guides = torch.zeros(20 * 20 * 4, dtype=torch.uint8, device=DEV)
    flags = torch.full((2,), -1, dtype=torch.int32, device=DEV)
    code = N.library().ssg_stage_images_resized(src.data_ptr(), 33, 35, 1, 2, 20, 20, N.ints([0]), 1,
                                               staged.data_ptr(), guides.data_ptr(), flags.data_ptr(),
                                               torch.cuda.current_stream().cuda_stream)
    assert code == N.SSG_ERR_UNSUPPORTED
    torch.cuda.synchronize()
    assert flags.cpu().tolist() == [-1, -1]


def _rig(ss, synthetic, width, cams_n=4, refs=(1, 3), seed=17, src=None):
    rng = np.random.Generator(np.random.PCG64(synthetic.frame_seed(7, seed)))
    cams = synthetic.ring_rig(rng, width, cams_n)
    scene = synthetic.random_scene(rng)
    src = src or (width, width)
    frame = synthetic.render_frame(scene, cams, src, src, list(refs))
    calibs = ss.parse_json_calib(synthetic.basalt_calibration(cams), (width, width), DEV)
    vp = torch.zeros(3, device=DEV)
    for r in refs:
        vp += calibs[r].rt[:3, 3] / len(refs)
    masks = [torch.ones(1, width, width, device=DEV) for _ in cams]
    return calibs, vp, masks, frame


@pytest.mark.parametrize("src_width", [304, 301])
@pytest.mark.parametrize("graphs", [False, True])
def test_pipeline_decoded_inputs_equal_resized_inputs(ss, native, synthetic, src_width, graphs):
    """The batched pipeline fed the decoded 8-bit renders (src_width^2, resized to 256^2 while
    staging; 301^2 has a pixel count the one-pass kernel declines, so the pipeline resizes first)
    gives the outputs it gives for the same renders resized to float32 beforehand, bit for bit."""
    width, refs = 256, [1, 3]
    calibs, vp, masks, frame = _rig(ss, synthetic, width, refs=refs, src=(src_width, src_width))
    decoded = torch.as_tensor(np.stack(frame.images_to_match), device=DEV)[None].repeat(2, 1, 1, 1, 1).contiguous()
    decoded[1] = decoded[1].flip(2)  # a second, different frame
    resized = ss.utils.resize_linear(decoded.view(-1, src_width, src_width, 3), (width, width))
    resized = resized.view(2, len(calibs), width, width, 3).contiguous()
    stitch = decoded[:, refs].contiguous()
    outs = []
    for match in (resized, decoded):
        est = ss.RGBD_Estimator(calibs, 0.55, 100.0, 32, refs, vp, masks, (width, width), (src_width, src_width),
                                (2 * width, width), 10.0, 6.25, DEV, cost_storage="fp16", max_batch=2,
                                cuda_graphs=graphs)
        for _ in range(2):  # the second run replays the captured graph
            rgb, dist = est.estimate_RGBD_panoramas(match, stitch)
        torch.cuda.synchronize()
        pipe = est.pipeline()
        outs.append((rgb.cpu().numpy(), dist.cpu().numpy(), est.batch_index_maps.cpu().numpy(),
                     pipe.plane_flags.cpu().numpy()))
        assert (pipe.plane_flags.cpu().numpy() == 1).all()  # resized renders hold fractions: 8.8 entries
    for a, b in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("dtype", ["float32", "uint8"])
@pytest.mark.parametrize("cols,rows", [(1024, 1024), (37, 50), (130, 70)])
def test_column_staging_equals_tile_staging(ss, native, dtype, cols, rows):
    """ssg_stage_images / ssg_stage_images_u8: the column-strip kernel gives the tile kernel's
    entries, guides and plane classes bit for bit (integer, fractional and out-of-range values)."""
    N = ss._native
    rng = np.random.default_rng(cols * rows)
    F, C, refs = 2, 3, [0, 2]
    imgs = rng.integers(0, 256, (F, C, rows, cols, 3)).astype(np.float32)
    if dtype == "float32":
        imgs[0, 1] += rng.uniform(-0.49, 0.49, imgs[0, 1].shape).astype(np.float32)
        imgs[0, 1] = np.clip(imgs[0, 1], 0, 255)
        imgs[1, 2, rows // 2, cols // 3, 1] = -3.0
        src = torch.as_tensor(imgs, device=DEV)
        entry = "ssg_stage_images"
    else:
        src = torch.as_tensor(imgs.astype(np.uint8), device=DEV)
        entry = "ssg_stage_images_u8"
    plane = (rows + 2) * (cols + 2)
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    try:
        for columns in (0, 1):
            N.call("ssg_tuning_set", N.TUNE_STAGE_COLUMNS, columns)
            staged = torch.full((F * C * 2 * plane * 4,), 7.0, device=DEV)
            guides = torch.zeros(F * len(refs) * rows * cols * 4, dtype=torch.uint8, device=DEV)
            flags = torch.full((F * C,), -1, dtype=torch.int32, device=DEV)
            N.call(entry, src.data_ptr(), F, C, cols, rows, N.ints(refs), len(refs), staged.data_ptr(),
                   guides.data_ptr(), flags.data_ptr(), stream)
            torch.cuda.synchronize()
            out.append((staged.cpu().numpy().view(np.uint32), guides.cpu().numpy(), flags.cpu().numpy()))
    finally:
        N.call("ssg_tuning_set", N.TUNE_STAGE_COLUMNS, 1)
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)
    if dtype == "float32":
        assert out[0][2].tolist() == [0, 1, 0, 0, 0, 2]


@pytest.mark.parametrize("graphs", [False, True])
def test_stitch_from_the_decoded_batch(ss, native, synthetic, graphs):
    """estimate_RGBD_panoramas(decoded) without images to stitch stitches the references' decoded
    images in place: the same panoramas bit for bit as passing those images explicitly."""
    width, refs, src_width = 256, [1, 3], 304
    calibs, vp, masks, frame = _rig(ss, synthetic, width, refs=refs, src=(src_width, src_width))
    decoded = torch.as_tensor(np.stack(frame.images_to_match), device=DEV)[None].repeat(2, 1, 1, 1, 1).contiguous()
    decoded[1] = decoded[1].flip(1)
    est = ss.RGBD_Estimator(calibs, 0.55, 100.0, 32, refs, vp, masks, (width, width), (src_width, src_width),
                            (2 * width, width), 10.0, 6.25, DEV, cost_storage="fp16", max_batch=2, cuda_graphs=graphs)
    rgb, dist = (t.clone() for t in est.estimate_RGBD_panoramas(decoded, decoded[:, refs].contiguous()))
    for _ in range(2):  # the second run replays the captured graph
        rgb2, dist2 = est.estimate_RGBD_panoramas(decoded)
    torch.cuda.synchronize()
    assert torch.equal(rgb2, rgb) and torch.equal(dist2, dist)
    # only decoded uint8 images at the stitch resolution can stand in for the images to stitch
    with pytest.raises(ValueError):
        est.estimate_RGBD_panoramas(decoded.float())
    small = ss.utils.resize_linear(decoded.view(-1, src_width, src_width, 3), (width, width), torch.uint8)
    with pytest.raises(ValueError):
        est.estimate_RGBD_panoramas(small.view(2, 4, width, width, 3).contiguous())

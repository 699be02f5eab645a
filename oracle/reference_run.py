"""Test infrastructure (oracle pinning only): run the reference implementation itself on CPU.

Imports the reference's own modules (python/utils.py, python/isb_filter.py, python/stitcher.py,
python/depth_estimation.py) from a reference checkout with three stand-ins:

* ``cupy`` -> oracle/fake_cupy.py (kernels compiled for the host from the reference's own .cu
  sources, with the fixed race-free schedule described in oracle/refcuda_harness_stitch.inc);
* ``cv2``, ``skimage``, ``skimage.metrics`` -> empty modules (only used by the reference's file
  I/O and evaluation, python/utils.py:157-250, which are not on the path).

``run_pipeline`` then follows python/main.py:63-112 with ``device='cpu'`` and records the
intermediate results of ``RGBD_Estimator.estimate_RGBD_panorama`` (cost volume before and after
the ISB filter, distance before and after the post-filter, stitcher tables) by wrapping the
instance's filter and stitcher methods; no reference code is modified.

Only tests/golden/make_golden.py uses this module, in a container that has the reference tree.
"""
from __future__ import annotations

import contextlib
import os
import sys
import types

import numpy as np
import torch

REFERENCE_ENV = "SPHERE_STEREO_REFERENCE"


def reference_root() -> str:
    """The reference checkout named by $SPHERE_STEREO_REFERENCE (a directory holding python/)."""
    root = os.environ.get(REFERENCE_ENV)
    if not root or not os.path.isdir(os.path.join(root, "python")):
        raise RuntimeError(f"set {REFERENCE_ENV} to a checkout of the reference (a directory with python/*.py)")
    return root


@contextlib.contextmanager
def _cwd(path):
    old = os.getcwd()
    os.chdir(path)
    try:
        yield
    finally:
        os.chdir(old)


def import_reference(reference_root: str):
    """Import the reference modules; returns a namespace with utils, isb_filter, stitcher,
    depth_estimation.  The kernel sources are read relative to the reference root."""
    here = os.path.dirname(os.path.abspath(__file__))
    if here not in sys.path:
        sys.path.insert(0, here)
    import fake_cupy

    sys.modules["cupy"] = fake_cupy
    for name in ("cv2", "skimage", "skimage.metrics"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["skimage.metrics"].structural_similarity = None
    sys.modules["skimage.metrics"].peak_signal_noise_ratio = None
    sys.modules["skimage"].metrics = sys.modules["skimage.metrics"]
    pydir = os.path.join(reference_root, "python")
    if pydir not in sys.path:
        sys.path.insert(0, pydir)
    with _cwd(reference_root):
        import utils  # noqa: F401  (reference module)
        import isb_filter
        import stitcher
        import depth_estimation
    return types.SimpleNamespace(utils=sys.modules["utils"], isb_filter=isb_filter, stitcher=stitcher,
                                 depth_estimation=depth_estimation, root=reference_root)


def run_isb_filter(ref, guide: np.ndarray, cost: np.ndarray, sigma_i: float, sigma_s: float):
    """``ISB_Filter(N, (cols, rows), 'cpu').apply(guide, cost, sigma_i, sigma_s)``."""
    n, rows, cols = cost.shape
    with _cwd(ref.root):
        filt = ref.isb_filter.ISB_Filter(n, (cols, rows), "cpu")
    g = torch.from_numpy(guide.copy())
    c = torch.from_numpy(cost.copy())
    out_cost, out_guide = filt.apply(g, c, sigma_i, sigma_s)
    return out_cost.numpy().copy(), out_guide.numpy().copy(), filt.scale_count


def run_pipeline(ref, calibration: dict, images_to_match, images_to_stitch, masks, *, min_dist, max_dist,
                 candidate_count, references_indices, matching_resolution, rgb_to_stitch_resolution,
                 panorama_resolution, sigma_i, sigma_s):
    """The reference's per-frame path on CPU (python/main.py:63-112); returns outputs and the
    recorded intermediates as numpy arrays."""
    utils, de = ref.utils, ref.depth_estimation
    device = "cpu"
    calibs = utils.parse_json_calib(calibration, list(matching_resolution), device)
    viewpoint = torch.zeros([3], device=device)
    for r in references_indices:
        viewpoint += calibs[r].rt[:3, 3] / len(references_indices)
    mask_t = [torch.tensor(m, dtype=torch.float32).unsqueeze(0) for m in masks]
    with _cwd(ref.root):
        est = de.RGBD_Estimator(calibs, min_dist, max_dist, candidate_count, list(references_indices), viewpoint,
                                mask_t, list(matching_resolution), list(rgb_to_stitch_resolution),
                                list(panorama_resolution), sigma_i, sigma_s, device)

    rec = {"guide": [], "cost_raw": [], "cost_filtered": [], "distance_raw": [], "distance_filtered": [],
           "guide_filtered_cost": [], "guide_filtered_distance": [], "index": []}
    cost_apply, dist_apply = est.cost_filter.apply, est.distance_filter.apply

    def cost_wrap(guide, cost, si, ss):
        rec["guide"].append(guide.numpy().copy())
        rec["cost_raw"].append(cost.numpy().copy())
        c, g = cost_apply(guide, cost, si, ss)
        rec["cost_filtered"].append(c.numpy().copy())
        # the selected candidate index, by the reference's own reduction (depth_estimation.py:180)
        rec["index"].append(torch.min(c, dim=0, keepdim=True)[1][0].numpy().astype(np.int16))
        rec["guide_filtered_cost"].append(g.numpy().copy())
        return c, g

    def dist_wrap(guide, dist, si, ss):
        rec["distance_raw"].append(dist.numpy().copy())
        d, g = dist_apply(guide, dist, si, ss)
        rec["distance_filtered"].append(d.numpy()[0].copy())
        rec["guide_filtered_distance"].append(g.numpy().copy())
        return d, g

    est.cost_filter.apply = cost_wrap
    est.distance_filter.apply = dist_wrap

    match_t = [torch.tensor(im, dtype=torch.float32) for im in images_to_match]
    stitch_t = [torch.tensor(im, dtype=torch.float32) for im in images_to_stitch]
    rgb, distance = est.estimate_RGBD_panorama(match_t, stitch_t)
    st = est.fishey_stitcher
    out = {
        "rgb_panorama": rgb.numpy().copy(),
        "distance_panorama": distance.numpy().copy(),
        "selected_cameras": np.stack([s[0].numpy() for s in est.selected_cameras]).astype(np.int8),
        "candidates": (1 / torch.linspace(1 / min_dist, 1 / max_dist, candidate_count)).numpy(),
        "reprojected_distances": st.reprojected_distances.numpy().copy(),
        "inpainting_tables": np.stack([w.numpy() for w in st.inpainting_weights_list]),
        "blending_sampling": st.blending_sampling.numpy().copy(),
        "blending_weights": st.blending_weights.numpy()[:, 0].copy(),
        "translations": st.translations.numpy().copy(),
        "calibration_vectors": st.calibration_vectors.numpy().copy(),
        "viewpoint": viewpoint.numpy().copy(),
        # rows 0..2 of inverse(camera.rt) @ reference.rt as the reference computes them
        # (depth_estimation.py:156), per reference and camera
        "relative_poses": np.stack([np.stack([torch.matmul(torch.inverse(c.rt), calibs[r].rt)[:3].reshape(12).numpy()
                                              for c in calibs]) for r in references_indices]),
    }
    for k, v in rec.items():
        out[k] = np.stack(v)
    return out


def build_reference_libraries(reference_root: str, candidate_counts=(1, 3, 8, 32)) -> None:
    """Compile the reference's kernels for the host into oracle/_ref (cached by content hash):
    the ISB module for each candidate count of the golden vectors, and the stitcher module of
    the small golden configuration.  The reference's own classes assemble the sources
    (python/isb_filter.py:47-52, python/stitcher.py:82-93); only the compiler is swapped."""
    import json

    ref = import_reference(reference_root)
    with _cwd(ref.root):
        for n in candidate_counts:
            ref.isb_filter.ISB_Filter(n, (16, 16), "cpu")
    here = os.path.dirname(os.path.abspath(__file__))
    golden = os.path.join(os.path.dirname(here), "tests", "golden", "pipeline_small.npz")
    if os.path.exists(golden):
        g = np.load(golden)
        cfg = json.loads(str(g["config"]))
        calibs = ref.utils.parse_json_calib(json.loads(str(g["calibration"])), cfg["matching_resolution"], "cpu")
        refs = cfg["references_indices"]
        viewpoint = torch.zeros(3)
        for r in refs:
            viewpoint += calibs[r].rt[:3, 3] / len(refs)
        masks = [torch.tensor(g["masks"][r])[None] for r in refs]
        with _cwd(ref.root):
            ref.stitcher.Stitcher([calibs[r] for r in refs], viewpoint, masks, cfg["min_dist"], cfg["max_dist"],
                                  cfg["matching_resolution"], cfg["rgb_to_stitch_resolution"],
                                  cfg["panorama_resolution"], "cpu")

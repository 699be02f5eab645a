"""Generate the golden vectors in tests/golden/ by running the reference implementation itself.

Needs a checkout of the reference, named by the environment variable SPHERE_STEREO_REFERENCE.
The reference's own Python (python/depth_estimation.py, python/isb_filter.py, python/stitcher.py,
python/utils.py) runs unmodified on CPU tensors; its two CUDA kernel files are compiled for the
host (oracle/fake_cupy.py, oracle/refcuda_shim.h, oracle/refcuda_harness_*.inc).  Inputs come
from the seeded synthetic rig and scene generator.

Fixtures written:
  isb_cases.npz       ISB_Filter.apply on random guides / costs: odd and even sizes, N in {1, 3, 32}
  pipeline_small.npz  a full frame at 90 x 75 matching (odd pyramid sizes), N = 8, circular masks,
                      with every intermediate of the reference
  pipeline_c1.npz     the 256^2 / N = 32 / 1024 x 512 panorama configuration, all-ones masks:
                      inputs, panorama outputs, per-reference guides, camera selections and
                      distance maps before and after the post-filter
  pipeline_c2.npz     the benchmarked prototype configuration: 1216^2 uint8 renders (frame 0 of
                      the benchmark's seeds), images to match resized to 1024^2 in float32 by
                      the linear resize the benchmark uses (so they hold fractions), N = 32,
                      sigma_s 25, references 2 and 3, stitch 1216^2, panorama 2048 x 1024.  The
                      inputs are not stored (48 MB): the fixture keeps their SHA-256 digests and
                      the tests regenerate them from the seed.  Camera selections and candidate
                      indices are stored whole; distances and panorama pixels on a 1/8 lattice
                      sample of the pixels, (x + 3 y) mod 8 == 0 (the acceptance statistics
                      are means over pixels).

Run:  SPHERE_STEREO_REFERENCE=<reference checkout> python tests/golden/make_golden.py [name ...]
      (names: isb small c1 c2; default all)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "sphere-stereo_gb300"))

import prep_eval_oracle  # noqa: E402
import reference_run  # noqa: E402
import synthetic  # noqa: E402

# (name, rows, cols, candidates, sigma_i, sigma_s, seed)
ISB_CASES = [
    ("odd_37x29_n3", 29, 37, 3, 10.0, 25.0, 11),
    ("even_64x48_n1", 48, 64, 1, 5.0, 12.5, 12),
    ("odd_33x21_n32", 21, 33, 32, 10.0, 6.25, 13),
    ("tall_40x71_n3", 71, 40, 3, 3.0, 40.0, 14),
]

SMALL = dict(width_in=180, height_in=150, matching=(90, 75), stitch=(120, 100), panorama=(128, 64),
             candidates=8, refs=[2, 3], sigma_i=10.0, sigma_s=6.25, seed=7, mask="circle")
C1 = dict(width_in=512, height_in=512, matching=(256, 256), stitch=(512, 512), panorama=(1024, 512),
          candidates=32, refs=[2, 3], sigma_i=10.0, sigma_s=6.25, seed=synthetic.frame_seed(1, 0), mask="ones")


# the benchmark's workload, frame 0 (its seeds are synthetic.frame_seed(2, frame))
C2 = dict(width_in=1216, matching=(1024, 1024), stitch=(1216, 1216), panorama=(2048, 1024), candidates=32,
          refs=[2, 3], sigma_i=10.0, sigma_s=25.0, seed=synthetic.frame_seed(2, 0), sample_stride=8)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def c2_inputs(cfg=C2):
    """The uint8 renders of every camera at the input resolution, the images to match (those
    resized to the matching resolution in float32 by the linear resize restated in
    oracle/prep_eval_oracle.py, which the library's ssg_resize_linear matches bit for bit) and the
    images to stitch (the references' renders), as the benchmark makes them."""
    w = cfg["width_in"]
    cams = synthetic.square_rig(w)
    rng = np.random.Generator(np.random.PCG64(cfg["seed"]))
    fr = synthetic.render_frame(synthetic.random_scene(rng), cams, (w, w), (w, w), [])
    originals = np.stack(fr.images_to_match)
    match = np.ascontiguousarray(np.stack([prep_eval_oracle.resize_linear(im, cfg["matching"]) for im in originals]))
    stitch = np.stack([originals[r] for r in cfg["refs"]])
    return cams, originals, match, stitch


def sample_lattice(cols: int, rows: int, stride: int) -> np.ndarray:
    """Flat indices of the pixels (x, y) with (x + 3 y) mod stride == 0: 1/stride of the pixels,
    with a phase that moves from row to row (the tests rebuild the same set)."""
    y, x = np.divmod(np.arange(cols * rows, dtype=np.int64), cols)
    return np.nonzero((x + 3 * y) % stride == 0)[0].astype(np.int32)


def make_pipeline_c2(ref, cfg=C2):
    cams, originals, match, stitch = c2_inputs(cfg)
    mw, mh = cfg["matching"]
    masks = [np.ones((mh, mw), np.float32) for _ in cams]
    calibration = synthetic.basalt_calibration(cams)
    kw = dict(min_dist=0.55, max_dist=100.0, candidate_count=cfg["candidates"], references_indices=cfg["refs"],
              matching_resolution=cfg["matching"], rgb_to_stitch_resolution=cfg["stitch"],
              panorama_resolution=cfg["panorama"], sigma_i=cfg["sigma_i"], sigma_s=cfg["sigma_s"])
    res = reference_run.run_pipeline(ref, calibration, list(match), list(stitch), masks, **kw)
    pw, ph = cfg["panorama"]
    pix = sample_lattice(mw, mh, cfg["sample_stride"])
    pano = sample_lattice(pw, ph, cfg["sample_stride"])
    R = len(cfg["refs"])
    inputs = {"seed": cfg["seed"], "width_in": cfg["width_in"], "renders_sha256": digest(originals),
              "images_to_match_sha256": digest(match), "images_to_stitch_sha256": digest(stitch)}
    out = {
        "config": np.array(json.dumps({**kw, "references_indices": list(cfg["refs"])})),
        "calibration": np.array(json.dumps(calibration)),
        "inputs": np.array(json.dumps(inputs)),
        "sample_stride": np.array(cfg["sample_stride"]),
    }
    for k in ("selected_cameras", "candidates", "index", "translations", "calibration_vectors", "viewpoint",
              "relative_poses"):
        out["ref/" + k] = res[k]
    out["ref/distance_raw@sample"] = res["distance_raw"].reshape(R, -1)[:, pix]
    out["ref/distance_filtered@sample"] = res["distance_filtered"].reshape(R, -1)[:, pix]
    out["ref/rgb_panorama@sample"] = res["rgb_panorama"].reshape(-1, 3)[pano]
    out["ref/distance_panorama@sample"] = res["distance_panorama"].reshape(-1)[pano]
    np.savez_compressed(os.path.join(HERE, "pipeline_c2.npz"), **out)


def make_isb(ref):
    out = {}
    for name, rows, cols, n, si, ss, seed in ISB_CASES:
        rng = np.random.Generator(np.random.PCG64(seed))
        # piecewise-smooth guide with edges, so the range weights vary
        yy, xx = np.meshgrid(np.arange(rows), np.arange(cols), indexing="ij")
        base = (40 + 150 * ((xx // 7 + yy // 5) % 2))[..., None] + rng.integers(0, 30, (rows, cols, 3))
        guide = np.clip(base, 0, 255).astype(np.uint8)
        cost = (rng.random((n, rows, cols)) * 500).astype(np.float32)
        c, g, levels = reference_run.run_isb_filter(ref, guide, cost, si, ss)
        out[f"{name}/guide"] = guide
        out[f"{name}/cost"] = cost
        out[f"{name}/sigma"] = np.array([si, ss])
        out[f"{name}/filtered_cost"] = c
        out[f"{name}/filtered_guide"] = g
        out[f"{name}/levels"] = np.array(levels)
    np.savez_compressed(os.path.join(HERE, "isb_cases.npz"), **out)


def make_pipeline(ref, cfg, filename, keep_volumes):
    rng = np.random.Generator(np.random.PCG64(cfg["seed"]))
    scene = synthetic.random_scene(rng)
    cams = synthetic.square_rig(cfg["width_in"], cfg["height_in"])
    frame = synthetic.render_frame(scene, cams, cfg["matching"], cfg["stitch"], cfg["refs"])
    mw, mh = cfg["matching"]
    if cfg["mask"] == "circle":
        masks = [synthetic.circular_mask(mw, mh) for _ in cams]
    else:
        masks = [np.ones((mh, mw), np.float32) for _ in cams]
    calibration = synthetic.basalt_calibration(cams)
    kw = dict(min_dist=0.55, max_dist=100.0, candidate_count=cfg["candidates"], references_indices=cfg["refs"],
              matching_resolution=cfg["matching"], rgb_to_stitch_resolution=cfg["stitch"],
              panorama_resolution=cfg["panorama"], sigma_i=cfg["sigma_i"], sigma_s=cfg["sigma_s"])
    res = reference_run.run_pipeline(ref, calibration, frame.images_to_match, frame.images_to_stitch, masks, **kw)
    out = {
        "config": np.array(json.dumps({**kw, "references_indices": list(cfg["refs"])})),
        "calibration": np.array(json.dumps(calibration)),
        "images_to_match": np.stack(frame.images_to_match),
        "images_to_stitch": np.stack(frame.images_to_stitch),
        "masks": np.stack(masks),
    }
    keep = ["rgb_panorama", "distance_panorama", "selected_cameras", "candidates", "index", "distance_raw",
            "distance_filtered", "guide", "translations", "calibration_vectors", "viewpoint", "relative_poses"]
    if keep_volumes:
        keep += ["cost_raw", "cost_filtered", "blending_sampling", "guide_filtered_cost", "guide_filtered_distance",
                 "reprojected_distances", "blending_weights", "inpainting_tables"]
    for k in keep:
        out["ref/" + k] = res[k]
    np.savez_compressed(os.path.join(HERE, filename), **out)


def main(names):
    ref = reference_run.import_reference(reference_run.reference_root())
    names = set(names or ("isb", "small", "c1", "c2"))
    if "isb" in names:
        make_isb(ref)
    if "small" in names:
        make_pipeline(ref, SMALL, "pipeline_small.npz", keep_volumes=True)
    if "c1" in names:
        make_pipeline(ref, C1, "pipeline_c1.npz", keep_volumes=False)
    if "c2" in names:
        make_pipeline_c2(ref)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)) // 1024, "KiB")


if __name__ == "__main__":
    main(sys.argv[1:])

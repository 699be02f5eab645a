"""TEST INFRASTRUCTURE -- the CPU oracle.  Used only by tests/, the smoke check and the CPU
baseline of the benchmark, as the checker; the product package never imports it.

Python glue around oracle/sphere_oracle.c (the C restatement of the reference's per-frame path).
``OracleRig`` mirrors the reference's host code: calibration parsing (python/utils.py:96-142),
RGBD_Estimator construction (python/depth_estimation.py:39-81), camera selection (:83-135), the
per-frame loop (:205-242), ISB_Filter.apply (python/isb_filter.py:72-136) and the stitcher
(python/stitcher.py:49-220).  Small host-side matrices (rt products, inverses, translations)
are computed with torch on the CPU in the reference's own expressions.

``precision="f32"`` is the reference's arithmetic; ``precision="f64"`` is the same algorithm in
float64, the yardstick for error statements.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np
import torch
from scipy.spatial.transform import Rotation

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SOURCE = os.path.join(_HERE, "sphere_oracle.c")
CFLAGS = ["-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-std=c11"]
_LOCK = threading.Lock()
_LIBS: dict[str, ctypes.CDLL] = {}


def library_path(precision: str) -> str:
    return os.path.join(_BUILD, f"libsphere_oracle_{precision}.so")


def build(force: bool = False) -> list[str]:
    """Compile the f32 and f64 oracle libraries into oracle/_build (gcc, a few seconds)."""
    os.makedirs(_BUILD, exist_ok=True)
    out = []
    procs = []
    for precision, real in (("f32", "float"), ("f64", "double")):
        path = library_path(precision)
        out.append(path)
        if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(_SOURCE):
            tmp = f"{path}.{os.getpid()}.tmp"
            procs.append((subprocess.Popen(["gcc", *CFLAGS, f"-DREAL={real}", _SOURCE, "-o", tmp, "-lm"]), tmp, path))
    for p, tmp, path in procs:
        if p.wait() != 0:
            raise RuntimeError(f"building {path} failed")
        os.replace(tmp, path)
    return out


_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_D = ctypes.c_double


def _signatures(real):
    return {
        "sso_rgb2ycbcr": [_P, _L, _P],
        "sso_unproject_grid": [_I, _I, _P, _P, _P],
        "sso_select_camera": [_I, _I, _I, _P, _I, _P, _P, _D, _D, _P],
        "sso_sweep_cost": [_I, _I, _I, _P, _I, _P, _P, _P, _P, _I, _P],
        "sso_isb_down": [_P, _P, _I, _I, _P, _P, _I, _I, _I, real],
        "sso_isb_up": [_P, _P, _I, _I, _P, _P, _I, _I, _I, real, real, real],
        "sso_isb_scale_count": [_I, _I],
        "sso_isb_apply": [_P, _P, _I, _I, _I, _D, _D],
        "sso_select_distance": [_P, _I, _L, _P, _P, _P],
        "sso_inpainting_table": [_I, _I, _P, _P, _D, _D, _P],
        "sso_box_filter": [_P, _I, _I, _I, _D, _P],
        "sso_blending_lut": [_I, _I, _I, _I, _I, _P, _P, _P, _P, _D, _D, _P, _P],
        "sso_reproject": [_P, _P, _I, _I, _P, _P],
        "sso_inpaint": [_P, _P, _I, _I, _D, _I],
        "sso_merge": [_P, _P, _P, _P, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I, _P, _P],
        "sso_set_exp_mode": [_I],
        "sso_isb_operators": [_P, _I, _I, _D, _D, _P, _P, _P, _P, _P],
        "sso_cw_expf": [ctypes.c_float],
    }


def load(precision: str = "f32") -> ctypes.CDLL:
    with _LOCK:
        if precision in _LIBS:
            return _LIBS[precision]
        path = library_path(precision)
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(_SOURCE):
            build()
        lib = ctypes.CDLL(path)
        real = ctypes.c_float if precision == "f32" else ctypes.c_double
        for name, args in _signatures(real).items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = {"sso_isb_scale_count": ctypes.c_int, "sso_cw_expf": ctypes.c_float}.get(name)
        _LIBS[precision] = lib
        return lib


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


class Oracle:
    """Thin typed wrappers over the C functions for one precision."""

    def __init__(self, precision: str = "f32", exp_mode: str = "libm"):
        """exp_mode "libm": the exponential the reference's kernels use on the host (the default,
        pinned against the reference); "device": the library's Cody-Waite exponential, for
        bit-for-bit comparisons with the CUDA kernels."""
        self.precision = precision
        self.lib = load(precision)
        self.dtype = np.float32 if precision == "f32" else np.float64
        self.exp_mode = {"libm": 0, "device": 1}[exp_mode]

    def __getattribute__(self, name):
        # the exponential mode is process-global in the library: set it before every call
        if name in ("isb_apply", "blending_lut", "rig_init"):
            object.__getattribute__(self, "lib").sso_set_exp_mode(object.__getattribute__(self, "exp_mode"))
        return object.__getattribute__(self, name)

    def cw_expf(self, x: float) -> float:
        return self.lib.sso_cw_expf(x)

    def real(self, a) -> np.ndarray:
        return np.ascontiguousarray(a, dtype=self.dtype)

    def rgb2ycbcr(self, rgb: np.ndarray) -> np.ndarray:
        rgb = self.real(rgb)
        out = np.empty(rgb.shape[:-1] + (3,), np.uint8)
        self.lib.sso_rgb2ycbcr(_ptr(rgb), rgb.size // 3, _ptr(out))
        return out

    def unproject_grid(self, W, H, cam6):
        cam = np.ascontiguousarray(cam6, np.float64)
        rays = np.empty((H, W, 3), self.dtype)
        valid = np.empty((H, W), np.uint8)
        self.lib.sso_unproject_grid(W, H, _ptr(cam), _ptr(rays), _ptr(valid))
        return rays, valid.astype(bool)

    def select_camera(self, W, H, cams, ref, rts, masks, min_dist, max_dist):
        cams = np.ascontiguousarray(cams, np.float64)
        rts = np.ascontiguousarray(rts, np.float32)
        masks = self.real(masks)
        out = np.empty((H, W), np.int8)
        self.lib.sso_select_camera(W, H, len(cams), _ptr(cams), ref, _ptr(rts), _ptr(masks), min_dist, max_dist,
                                   _ptr(out))
        return out

    def sweep_cost(self, W, H, cams, ref, rts, images, selected, candidates):
        cams = np.ascontiguousarray(cams, np.float64)
        rts = np.ascontiguousarray(rts, np.float32)
        images = self.real(images)
        selected = np.ascontiguousarray(selected, np.int8)
        candidates = self.real(candidates)
        n = len(candidates)
        cost = np.empty((n, H, W), self.dtype)
        self.lib.sso_sweep_cost(W, H, len(cams), _ptr(cams), ref, _ptr(rts), _ptr(images), _ptr(selected),
                                _ptr(candidates), n, _ptr(cost))
        return cost

    def isb_apply(self, guide, cost, sigma_i, sigma_s):
        guide = np.ascontiguousarray(guide, np.uint8).copy()
        cost = self.real(cost).copy()
        n, rows, cols = cost.shape
        self.lib.sso_isb_apply(_ptr(guide), _ptr(cost), n, rows, cols, sigma_i, sigma_s)
        return cost, guide

    def isb_operators(self, guide, sigma_i, sigma_s):
        """The filter of isb_apply for this guide as explicit sparse operators (see
        sso_isb_operators): dict with per-level lists down_idx/down_w ([P_s, 9], s >= 1) and
        up_idx/up_w ([P_s, 9]) / up_own ([P_s]) (s <= L - 2), plus the level shapes."""
        self.lib.sso_set_exp_mode(self.exp_mode)
        guide = np.ascontiguousarray(guide, np.uint8)
        rows, cols = guide.shape[:2]
        L = self.isb_scale_count(cols, rows)
        shapes = [(int(math.ceil(rows / 2 ** s)), int(math.ceil(cols / 2 ** s))) for s in range(L)]
        di = [np.zeros((max(1, r * c), 9), np.int32) for r, c in shapes]
        dw = [np.zeros((max(1, r * c), 9), self.dtype) for r, c in shapes]
        ui = [np.zeros((max(1, r * c), 9), np.int32) for r, c in shapes]
        uw = [np.zeros((max(1, r * c), 9), self.dtype) for r, c in shapes]
        uo = [np.zeros((max(1, r * c),), self.dtype) for r, c in shapes]
        arr = lambda xs: (ctypes.c_void_p * len(xs))(*[x.ctypes.data for x in xs])  # noqa: E731
        self.lib.sso_isb_operators(_ptr(guide), rows, cols, sigma_i, sigma_s, arr(di), arr(dw), arr(ui), arr(uw),
                                   arr(uo))
        return {"shapes": shapes, "down_idx": di, "down_w": dw, "up_idx": ui, "up_w": uw, "up_own": uo}

    def isb_scale_count(self, cols, rows):
        return self.lib.sso_isb_scale_count(cols, rows)

    def select_distance(self, cost, candidates):
        cost = self.real(cost)
        n = cost.shape[0]
        p = cost[0].size
        candidates = self.real(candidates)
        dist = np.empty(cost.shape[1:], self.dtype)
        index = np.empty(cost.shape[1:], np.int32)
        self.lib.sso_select_distance(_ptr(cost), n, p, _ptr(candidates), _ptr(dist), _ptr(index))
        return dist, index

    def inpainting_table(self, W, H, k6, t3, min_dist, max_dist):
        k6 = np.ascontiguousarray(k6, np.float32)
        t3 = np.ascontiguousarray(t3, np.float32)
        out = np.empty((H, W, 2), np.uint8)
        self.lib.sso_inpainting_table(W, H, _ptr(k6), _ptr(t3), min_dist, max_dist, _ptr(out))
        return out

    def box_filter(self, img, radius, pad_value):
        img = self.real(img)
        out = np.empty_like(img)
        H, W = img.shape
        self.lib.sso_box_filter(_ptr(img), H, W, radius, pad_value, _ptr(out))
        return out

    def blending_lut(self, W, H, Wp, Hp, ks, rots, ts, masks_filtered, min_dist, max_dist):
        R = len(ks)
        ks = np.ascontiguousarray(ks, np.float32)
        rots = np.ascontiguousarray(rots, np.float32)
        ts = np.ascontiguousarray(ts, np.float32)
        masks_filtered = self.real(masks_filtered)
        lut = np.empty((R, Hp, Wp, 2), self.dtype)
        weights = np.empty((R, Hp, Wp), self.dtype)
        self.lib.sso_blending_lut(W, H, Wp, Hp, R, _ptr(ks), _ptr(rots), _ptr(ts), _ptr(masks_filtered), min_dist,
                                  max_dist, _ptr(lut), _ptr(weights))
        return lut, weights

    def reproject(self, dist, k6, t3, fill=1e8):
        dist = self.real(dist)
        H, W = dist.shape
        out = np.full((H, W), fill, self.dtype)
        self.lib.sso_reproject(_ptr(dist), _ptr(out), W, H, _ptr(np.ascontiguousarray(k6, np.float32)),
                               _ptr(np.ascontiguousarray(t3, np.float32)))
        return out

    def inpaint(self, dist, table, max_dist, iterations):
        dist = self.real(dist).copy()
        H, W = dist.shape
        self.lib.sso_inpaint(_ptr(dist), _ptr(np.ascontiguousarray(table, np.uint8)), W, H, max_dist, iterations)
        return dist

    def merge(self, lut, weights, reproj, dists, images, ts, ks):
        R, Hp, Wp = weights.shape
        _, H, W = reproj.shape
        images = np.ascontiguousarray(images, np.uint8)
        Hs, Ws = images.shape[1], images.shape[2]
        dist = np.empty((Hp, Wp), self.dtype)
        rgb = np.empty((Hp, Wp, 3), np.uint8)
        self.lib.sso_merge(_ptr(self.real(lut)), _ptr(self.real(weights)), _ptr(self.real(reproj)),
                           _ptr(self.real(dists)), _ptr(images), Hs, Ws,
                           _ptr(np.ascontiguousarray(ts, np.float32)), _ptr(np.ascontiguousarray(ks, np.float32)),
                           R, W, H, Wp, Hp, _ptr(dist), _ptr(rgb))
        return dist, rgb


# ---------------------------------------------------------------------------------------------
# Host-side calibration math, in the reference's torch expressions (CPU, float32 or float64)
# ---------------------------------------------------------------------------------------------

def parse_calibration(raw: dict, matching_resolution, dtype=torch.float32):
    """python/utils.py:96-142 -> list of dicts with rt (4x4), fl, principal, matching_scale
    (torch tensors of ``dtype``) and xi, alpha (Python floats)."""
    cams = []
    for ext, intr, res in zip(raw["T_imu_cam"], raw["intrinsics"], raw["resolution"]):
        if intr["camera_type"] != "ds":
            raise Exception("Unexpected camera model. The current implementation only support double sphere.")
        ci = intr["intrinsics"]
        r = Rotation.from_quat([ext["qx"], ext["qy"], ext["qz"], ext["qw"]])
        rt = torch.eye(4, dtype=dtype)
        rt[:3, :3] = torch.tensor(r.as_matrix(), dtype=torch.float64).to(dtype)
        rt[:3, 3] = torch.tensor([ext["px"], ext["py"], ext["pz"]], dtype=dtype)
        cams.append({
            "rt": rt,
            "fl": torch.tensor([ci["fx"], ci["fy"]], dtype=dtype),
            "principal": torch.tensor([ci["cx"], ci["cy"]], dtype=dtype),
            "xi": ci["xi"], "alpha": ci["alpha"],
            "matching_scale": torch.tensor([matching_resolution[0] / res[0], matching_resolution[1] / res[1]],
                                           dtype=dtype),
        })
    return cams


def cam6(cam) -> np.ndarray:
    """{fl * s, principal * s} in the calibration dtype plus xi, alpha as Python floats."""
    fs = (cam["fl"] * cam["matching_scale"]).double().numpy()
    ps = (cam["principal"] * cam["matching_scale"]).double().numpy()
    return np.array([fs[0], fs[1], ps[0], ps[1], cam["xi"], cam["alpha"]], np.float64)


def intrinsics_vector(cam) -> np.ndarray:
    """vectorize_calibration (python/stitcher.py:35-46): float32 [fx*s, fy*s, cx*s, cy*s, xi, alpha]."""
    v = torch.zeros(6, dtype=torch.float32)
    v[0:2] = (cam["fl"] * cam["matching_scale"]).float()
    v[2:4] = (cam["principal"] * cam["matching_scale"]).float()
    v[4] = cam["xi"]
    v[5] = cam["alpha"]
    return v.numpy()


def relative_rts(cams, ref: int) -> np.ndarray:
    """rows 0..2 of torch.matmul(torch.inverse(cam.rt), ref.rt) per camera
    (python/depth_estimation.py:104,156), C x 12."""
    out = [torch.matmul(torch.inverse(c["rt"]), cams[ref]["rt"])[:3].reshape(12) for c in cams]
    return torch.stack(out).double().numpy()


class OracleRig:
    """The reference's per-rig state and per-frame path, on the C oracle."""

    def __init__(self, calibration: dict, *, min_dist, max_dist, candidate_count, references_indices, masks,
                 matching_resolution, rgb_to_stitch_resolution, panorama_resolution, sigma_i, sigma_s,
                 precision="f32", smoothing_radius=15, inpainting_iterations=32, exp_mode="libm"):
        self.o = Oracle(precision, exp_mode)
        tdtype = torch.float32 if precision == "f32" else torch.float64
        self.tdtype = tdtype
        self.cams = parse_calibration(calibration, matching_resolution, tdtype)
        self.W, self.H = matching_resolution
        self.Ws, self.Hs = rgb_to_stitch_resolution
        self.Wp, self.Hp = panorama_resolution
        self.min_dist, self.max_dist = float(min_dist), float(max_dist)
        self.N = candidate_count
        self.refs = list(references_indices)
        self.sigma_i, self.sigma_s = sigma_i, sigma_s
        self.iterations = inpainting_iterations
        self.cam6 = np.stack([cam6(c) for c in self.cams])
        self.masks = np.stack([np.asarray(m, np.float64).reshape(self.H, self.W) for m in masks])
        self.candidates = (1 / torch.linspace(1 / self.min_dist, 1 / self.max_dist, self.N, dtype=tdtype)).numpy()
        self.rts = {r: relative_rts(self.cams, r) for r in self.refs}
        self.selected = {r: self.o.select_camera(self.W, self.H, self.cam6, r, self.rts[r], self.masks,
                                                 self.min_dist, self.max_dist) for r in self.refs}
        # stitcher tables (python/stitcher.py:75-164)
        vp = torch.zeros(3, dtype=tdtype)
        for r in self.refs:
            vp += self.cams[r]["rt"][:3, 3] / len(self.refs)
        self.viewpoint = vp.numpy()
        vp4 = torch.cat([vp, torch.ones(1, dtype=tdtype)])
        self.ks = np.stack([intrinsics_vector(self.cams[r]) for r in self.refs])
        self.ts = np.stack([torch.matmul(torch.inverse(self.cams[r]["rt"]), vp4)[:3].float().numpy()
                            for r in self.refs])
        self.rots = np.stack([torch.inverse(self.cams[r]["rt"][:3, :3]).float().reshape(9).numpy() for r in self.refs])
        self.tables = np.stack([self.o.inpainting_table(self.W, self.H, k, t, self.min_dist, self.max_dist)
                                for k, t in zip(self.ks, self.ts)])
        masks_f = np.stack([self.o.box_filter(self.masks[r], smoothing_radius, 1.0) for r in self.refs])
        self.masks_filtered = masks_f
        lut, weights = self.o.blending_lut(self.W, self.H, self.Wp, self.Hp, self.ks, self.rots, self.ts, masks_f,
                                           self.min_dist, self.max_dist)
        weights = np.stack([self.o.box_filter(w, smoothing_radius, 0.0) for w in weights])
        self.blending_lut = lut
        self.blending_weights = (weights / weights.sum(axis=0, keepdims=True)).astype(self.o.dtype)

    def set_rig_tables(self, selected_cameras=None, relative_poses=None):
        """Use another run's camera-selection maps ([references][rows, cols]) and relative poses
        ([references][cameras, 12]) instead of this host's (see RGBD_Estimator.set_rig_tables)."""
        if selected_cameras is not None:
            for r, s in zip(self.refs, selected_cameras):
                self.selected[r] = np.ascontiguousarray(s, np.int8).reshape(self.H, self.W)
        if relative_poses is not None:
            for r, p in zip(self.refs, relative_poses):
                self.rts[r] = np.asarray(p, np.float64).reshape(-1, 12)

    def estimate(self, images_to_match, images_to_stitch, keep_intermediates=False):
        """estimate_RGBD_panorama (python/depth_estimation.py:205-242) on the oracle."""
        images = np.stack([np.asarray(im) for im in images_to_match]).astype(self.o.dtype)
        rec = {"guide": [], "cost_raw": [], "cost_filtered": [], "distance_raw": [], "distance_filtered": [],
               "index": []}
        for r in self.refs:
            guide = self.o.rgb2ycbcr(images[r])
            cost = self.o.sweep_cost(self.W, self.H, self.cam6, r, self.rts[r], images, self.selected[r],
                                     self.candidates)
            fcost, _ = self.o.isb_apply(guide, cost, self.sigma_i, self.sigma_s)
            dist, index = self.o.select_distance(fcost, self.candidates)
            fdist, _ = self.o.isb_apply(guide, dist[None], self.sigma_i / 2, self.sigma_s / 2)
            rec["distance_filtered"].append(fdist[0])
            if keep_intermediates:
                rec["guide"].append(guide)
                rec["cost_raw"].append(cost)
                rec["cost_filtered"].append(fcost)
                rec["distance_raw"].append(dist)
                rec["index"].append(index)
        stitch = np.stack([np.asarray(im) for im in images_to_stitch]).astype(np.float32).astype(np.uint8)
        dists = np.stack(rec["distance_filtered"])
        reproj = np.stack([self.o.inpaint(self.o.reproject(d, k, t), tab, self.max_dist, self.iterations)
                           for d, k, t, tab in zip(dists, self.ks, self.ts, self.tables)])
        dpano, rgb = self.o.merge(self.blending_lut, self.blending_weights, reproj, dists, stitch, self.ts, self.ks)
        out = {"rgb_panorama": rgb, "distance_panorama": dpano, "reprojected_distances": reproj,
               "distance_filtered": dists}
        if keep_intermediates:
            for k, v in rec.items():
                if k != "distance_filtered" and v:
                    out[k] = np.stack(v)
        return out

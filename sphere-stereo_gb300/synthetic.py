"""Seeded synthetic rigs and scenes: the stand-in for the reference's evaluation dataset.

The reference is evaluated on captured fisheye rigs (python/main.py:63-112 reads a basalt
calibration file plus one image per camera).  That dataset is not available here, so every
workload in this project is generated by this module instead:

* a rig of double-sphere fisheye cameras, written as a basalt-format calibration dictionary
  that ``parse_json_calib`` (python/utils.py:96-142) consumes unchanged;
* a 6 x 5 x 3 m box room (x: 6 m, z: 5 m, y: 3 m vertical, y pointing down like the camera
  and panorama conventions of python/stitcher.cu:349-354) with spheres of radius 0.2-1.0 m,
  textured with seeded solid value noise;
* a float64 ray caster producing uint8 RGB fisheye images and ground-truth inverse distance.

Everything is numpy float64 with integer hashing for the noise, so a seed gives the same
images on any host (up to libm differences in the few trigonometric calls of the rig).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

ROOM_HALF = np.array([3.0, 1.5, 2.5])  # half extents of the 6 (x) x 3 (y) x 5 (z) m room


@dataclass
class RigCamera:
    """One double-sphere camera: intrinsics at its native resolution and its camera->rig pose."""
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float
    xi: float
    alpha: float
    rotation: np.ndarray  # [3, 3] camera -> rig
    position: np.ndarray  # [3] camera centre in the rig frame

    def scaled(self, width: int, height: int) -> "RigCamera":
        """Intrinsics scaled to another image size, as ``matching_scale`` does in the reference."""
        sx, sy = width / self.width, height / self.height
        return RigCamera(width, height, self.fx * sx, self.fy * sy, self.cx * sx, self.cy * sy,
                         self.xi, self.alpha, self.rotation, self.position)


def rotation_y(theta: float) -> np.ndarray:
    c, s = math.cos(theta), math.sin(theta)
    return np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])


def rotation_axis_angle(axis: np.ndarray, angle: float) -> np.ndarray:
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + math.sin(angle) * k + (1 - math.cos(angle)) * (k @ k)


def matrix_to_quaternion(r: np.ndarray) -> tuple[float, float, float, float]:
    """Rotation matrix -> unit quaternion (x, y, z, w), Shepperd's method."""
    tr = r[0, 0] + r[1, 1] + r[2, 2]
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        w, x, y, z = 0.25 * s, (r[2, 1] - r[1, 2]) / s, (r[0, 2] - r[2, 0]) / s, (r[1, 0] - r[0, 1]) / s
    elif r[0, 0] > r[1, 1] and r[0, 0] > r[2, 2]:
        s = math.sqrt(1.0 + r[0, 0] - r[1, 1] - r[2, 2]) * 2
        w, x, y, z = (r[2, 1] - r[1, 2]) / s, 0.25 * s, (r[0, 1] + r[1, 0]) / s, (r[0, 2] + r[2, 0]) / s
    elif r[1, 1] > r[2, 2]:
        s = math.sqrt(1.0 + r[1, 1] - r[0, 0] - r[2, 2]) * 2
        w, x, y, z = (r[0, 2] - r[2, 0]) / s, (r[0, 1] + r[1, 0]) / s, 0.25 * s, (r[1, 2] + r[2, 1]) / s
    else:
        s = math.sqrt(1.0 + r[2, 2] - r[0, 0] - r[1, 1]) * 2
        w, x, y, z = (r[1, 0] - r[0, 1]) / s, (r[0, 2] + r[2, 0]) / s, (r[1, 2] + r[2, 1]) / s, 0.25 * s
    return x, y, z, w


def square_rig(width: int, height: int | None = None, xi: float = -0.2, alpha: float = 0.6,
               half_side: float = 0.1, count: int = 4) -> list[RigCamera]:
    """Four cameras at the corners (+-0.1, +-0.1) m of the horizontal x-z plane, optical axes
    pointing outward at 45 deg + k * 90 deg, fx = fy = 0.28 W, principal point at the centre."""
    height = width if height is None else height
    cams = []
    radius = half_side * math.sqrt(2.0)
    for k in range(count):
        theta = math.radians(45.0 + k * 360.0 / count)
        direction = np.array([math.sin(theta), 0.0, math.cos(theta)])
        cams.append(RigCamera(width, height, 0.28 * width, 0.28 * width, width / 2, height / 2,
                              xi, alpha, rotation_y(theta), radius * direction))
    return cams


def ring_rig(rng: np.random.Generator, width: int, count: int) -> list[RigCamera]:
    """A ring of ``count`` outward cameras, radius 0.1-0.3 m, xi in [-0.3, 0], alpha in [0.5, 0.7]."""
    radius = rng.uniform(0.1, 0.3)
    phase = rng.uniform(0, 2 * math.pi)
    cams = []
    for k in range(count):
        theta = phase + 2 * math.pi * k / count
        direction = np.array([math.sin(theta), 0.0, math.cos(theta)])
        cams.append(RigCamera(width, width, 0.28 * width, 0.28 * width, width / 2, width / 2,
                              float(rng.uniform(-0.3, 0.0)), float(rng.uniform(0.5, 0.7)),
                              rotation_y(theta), radius * direction))
    return cams


def perturb_rig(cams: list[RigCamera], rng: np.random.Generator, angle_deg: float = 0.5,
                translation: float = 0.005) -> list[RigCamera]:
    """Seeded extrinsic noise: a rotation of ``angle_deg`` about a random axis and a translation
    of ``translation`` metres in a random direction, per camera."""
    out = []
    for cam in cams:
        axis = rng.normal(size=3)
        dr = rotation_axis_angle(axis, math.radians(angle_deg))
        dt = rng.normal(size=3)
        dt = translation * dt / np.linalg.norm(dt)
        out.append(RigCamera(cam.width, cam.height, cam.fx, cam.fy, cam.cx, cam.cy, cam.xi, cam.alpha,
                             dr @ cam.rotation, cam.position + dt))
    return out


def basalt_calibration(cams: list[RigCamera]) -> dict:
    """The rig as the ``value0`` dictionary of a basalt calibration file (what
    python/main.py:63-65 passes to ``parse_json_calib``)."""
    t_imu_cam, intrinsics, resolution = [], [], []
    for cam in cams:
        qx, qy, qz, qw = matrix_to_quaternion(cam.rotation)
        t_imu_cam.append({"px": float(cam.position[0]), "py": float(cam.position[1]),
                          "pz": float(cam.position[2]), "qx": qx, "qy": qy, "qz": qz, "qw": qw})
        intrinsics.append({"camera_type": "ds", "intrinsics": {
            "fx": cam.fx, "fy": cam.fy, "cx": cam.cx, "cy": cam.cy, "xi": cam.xi, "alpha": cam.alpha}})
        resolution.append([cam.width, cam.height])
    return {"T_imu_cam": t_imu_cam, "intrinsics": intrinsics, "resolution": resolution}


# ---------------------------------------------------------------------------------------------
# Double-sphere model in float64 (the model of python/utils.py:57-94)
# ---------------------------------------------------------------------------------------------

def ds_unproject(u: np.ndarray, v: np.ndarray, cam: RigCamera) -> tuple[np.ndarray, np.ndarray]:
    mx = (u - cam.cx) / cam.fx
    my = (v - cam.cy) / cam.fy
    r2 = mx * mx + my * my
    a = cam.alpha
    disc = 1.0 - (2.0 * a - 1.0) * r2
    valid = disc >= 0
    mz = (1.0 - a * a * r2) / (a * np.sqrt(np.maximum(disc, 0.0)) + 1.0 - a)
    scale = (mz * cam.xi + np.sqrt(mz * mz + (1.0 - cam.xi * cam.xi) * r2)) / (mz * mz + r2)
    pts = np.stack([scale * mx, scale * my, scale * mz - cam.xi], axis=-1)
    return pts, valid


# ---------------------------------------------------------------------------------------------
# Scene and ray caster
# ---------------------------------------------------------------------------------------------

def _hash3(ix, iy, iz, seed: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) \
            ^ (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32((seed * 0x165667B1) & 0xFFFFFFFF)
        h ^= h >> np.uint32(13)
        h *= np.uint32(0x5BD1E995)
        h ^= h >> np.uint32(15)
        h *= np.uint32(0x27D4EB2F)
        h ^= h >> np.uint32(16)
    return h.astype(np.float64) * (1.0 / 4294967296.0)


def value_noise(p: np.ndarray, frequency: float, seed: int) -> np.ndarray:
    """Trilinearly interpolated lattice noise (smoothstep fade) in [0, 1)."""
    q = p * frequency
    f = np.floor(q)
    t = q - f
    t = t * t * (3.0 - 2.0 * t)
    i = f.astype(np.int64)
    out = 0.0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (t[..., 0] if dx else 1 - t[..., 0]) * (t[..., 1] if dy else 1 - t[..., 1]) \
                    * (t[..., 2] if dz else 1 - t[..., 2])
                out = out + w * _hash3(i[..., 0] + dx, i[..., 1] + dy, i[..., 2] + dz, seed)
    return out


@dataclass
class Scene:
    sphere_centres: np.ndarray  # [S, 3]
    sphere_radii: np.ndarray    # [S]
    colours: np.ndarray         # [S + 1, 3] base colours; last row is the room
    seed: int
    rig_centre: np.ndarray = field(default_factory=lambda: np.zeros(3))


def random_scene(rng: np.random.Generator, sphere_count: int = 20, rig_centre=None) -> Scene:
    """Spheres of radius U[0.2, 1.0] m with centres uniform inside the room, fully inside it and
    at least r + 0.6 m from the rig centre."""
    rig_centre = np.zeros(3) if rig_centre is None else np.asarray(rig_centre, dtype=np.float64)
    centres, radii = [], []
    while len(centres) < sphere_count:
        r = rng.uniform(0.2, 1.0)
        c = rng.uniform(-ROOM_HALF + r, ROOM_HALF - r)
        if np.linalg.norm(c - rig_centre) >= r + 0.6:
            centres.append(c)
            radii.append(r)
    colours = rng.uniform(0.25, 1.0, size=(sphere_count + 1, 3))
    return Scene(np.array(centres), np.array(radii), colours, int(rng.integers(0, 2**31 - 1)), rig_centre)


def cast(scene: Scene, origin: np.ndarray, dirs: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Nearest hit distance (along unit ``dirs``) and object id (sphere index, or S for the room)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        t_wall = np.full(dirs.shape[:-1], np.inf)
        for axis in range(3):
            d = dirs[..., axis]
            bound = np.where(d > 0, ROOM_HALF[axis], -ROOM_HALF[axis])
            t = (bound - origin[axis]) / d
            t_wall = np.minimum(t_wall, np.where(d != 0, t, np.inf))
    best_t = t_wall
    best_id = np.full(dirs.shape[:-1], len(scene.sphere_radii), dtype=np.int64)
    for s, (c, r) in enumerate(zip(scene.sphere_centres, scene.sphere_radii)):
        oc = origin - c
        b = dirs @ oc
        cc = float(oc @ oc - r * r)
        disc = b * b - cc
        hit = disc >= 0
        t = -b - np.sqrt(np.where(hit, disc, 0.0))
        hit &= (t > 1e-6) & (t < best_t)
        best_t = np.where(hit, t, best_t)
        best_id = np.where(hit, s, best_id)
    return best_t, best_id


def shade(scene: Scene, points: np.ndarray, ids: np.ndarray) -> np.ndarray:
    """Solid value-noise texture times the object's base colour, in [0, 255]."""
    n = 0.45 * value_noise(points, 3.0, scene.seed) + 0.35 * value_noise(points, 17.0, scene.seed + 1) \
        + 0.20 * value_noise(points, 61.0, scene.seed + 2)
    rgb = np.empty(points.shape[:-1] + (3,))
    for ch in range(3):
        nc = value_noise(points, 23.0, scene.seed + 11 + ch)
        rgb[..., ch] = scene.colours[ids, ch] * (0.2 + 0.8 * (0.75 * n + 0.25 * nc))
    return np.clip(rgb * 255.0, 0.0, 255.0)


def render_fisheye(scene: Scene, cam: RigCamera, width: int, height: int,
                   chunk_rows: int = 128) -> tuple[np.ndarray, np.ndarray]:
    """Ray-cast a [height, width, 3] uint8 image and its [height, width] ground-truth inverse
    distance (0 outside the double-sphere model's valid area) for ``cam`` rescaled to that size."""
    c = cam.scaled(width, height)
    image = np.zeros((height, width, 3), dtype=np.uint8)
    inv_distance = np.zeros((height, width), dtype=np.float64)
    for y0 in range(0, height, chunk_rows):
        y1 = min(height, y0 + chunk_rows)
        v, u = np.meshgrid(np.arange(y0, y1, dtype=np.float64), np.arange(width, dtype=np.float64), indexing="ij")
        rays, valid = ds_unproject(u, v, c)
        rays = rays / np.linalg.norm(rays, axis=-1, keepdims=True)
        dirs = rays @ c.rotation.T
        t, ids = cast(scene, c.position, dirs)
        pts = c.position + t[..., None] * dirs
        rgb = shade(scene, pts, ids)
        image[y0:y1] = np.where(valid[..., None], np.floor(rgb), 0).astype(np.uint8)
        inv_distance[y0:y1] = np.where(valid, 1.0 / t, 0.0)
    return image, inv_distance


def render_panorama_depth(scene: Scene, viewpoint: np.ndarray, width: int, height: int) -> np.ndarray:
    """Ground-truth inverse distance of the equirectangular panorama at ``viewpoint``, with the
    pixel->ray mapping of python/stitcher.cu:346-354."""
    y, x = np.meshgrid(np.arange(height, dtype=np.float64), np.arange(width, dtype=np.float64), indexing="ij")
    phi = (y + 0.5) * math.pi / height - math.pi / 2
    theta = (x + 0.5) * 2 * math.pi / width + math.pi
    dirs = np.stack([np.cos(phi) * np.sin(theta), np.sin(phi), np.cos(phi) * np.cos(theta)], axis=-1)
    t, _ = cast(scene, np.asarray(viewpoint, dtype=np.float64), dirs)
    return 1.0 / t


@dataclass
class Frame:
    images_to_match: list[np.ndarray]   # C x [H, W, 3] uint8
    images_to_stitch: list[np.ndarray]  # R x [Hs, Ws, 3] uint8
    inv_distance: list[np.ndarray]      # C x [H, W] float64 ground truth at matching resolution


def render_frame(scene: Scene, cams: list[RigCamera], matching_resolution, rgb_to_stitch_resolution,
                 references_indices) -> Frame:
    """All images of one frame; resolutions are (cols, rows) like the reference's arguments."""
    mw, mh = matching_resolution
    sw, sh = rgb_to_stitch_resolution
    match, inv = [], []
    for cam in cams:
        img, d = render_fisheye(scene, cam, mw, mh)
        match.append(img)
        inv.append(d)
    stitch = [render_fisheye(scene, cams[r], sw, sh)[0] for r in references_indices]
    return Frame(match, stitch, inv)


def frame_seed(config: int, frame: int) -> int:
    """Seed convention of the synthetic workloads: 1000 * config + frame."""
    return 1000 * config + frame


def circular_mask(width: int, height: int, radius_fraction: float = 0.47) -> np.ndarray:
    """A [height, width] float32 mask that is 1 inside a centred circle and 0 outside, with a
    one-pixel linear ramp so that the reference's mask thresholds (>= 0.9, > 0.99) are exercised."""
    y, x = np.meshgrid(np.arange(height) + 0.5, np.arange(width) + 0.5, indexing="ij")
    r = np.hypot(x - width / 2, y - height / 2)
    edge = radius_fraction * min(width, height)
    return np.clip(edge - r + 0.5, 0.0, 1.0).astype(np.float32)

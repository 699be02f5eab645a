"""ctypes binding of libsphere_stereo_gb300.so (the C ABI declared in include/sphere_stereo_gb300.h).

There is no fallback: if the library is missing or fails to load, every entry point raises
NativeLibraryError.  Device pointers are passed as integers (``tensor.data_ptr()``), streams as
``torch.cuda.current_stream().cuda_stream``.
"""
from __future__ import annotations

import ctypes
import math
import os
import threading

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY = os.path.join(HERE, "libsphere_stereo_gb300.so")

SSG_OK = 0
SSG_ERR_INVALID_ARGUMENT = 1
SSG_ERR_CUDA = 2
SSG_ERR_UNSUPPORTED = 3
MAX_CAMERAS = 16
MAX_CANDIDATES = 256
MAX_REFERENCES = 16
MAX_LEVELS = 24
TUNE_SWEEP_VARIANT = 0
TUNE_HOLE_BLOCKS_PER_SM = 1
TUNE_MERGE_FRAMES = 2
TUNE_UNEVEN_SPAN = 3
TUNE_ISB_UP_BLOCKS = 4
TUNE_ISB_SELECT_BLOCKS = 5
TUNE_ISB_TILE_TMA = 6
TUNE_TMA_WITHHOLD = 7
TUNE_HOLE_PERSISTENT = 8
TUNE_SWEEP_TILES = 9
TUNE_HOLE_TAIL = 10
TUNE_SELECT_WHOLE = 11
TUNE_UP_WHOLE = 12
TUNE_ISB_TAIL = 13
TUNE_POST_TAIL = 14
TUNE_STAGE_COLUMNS = 15
STATUS_TMA_TIMEOUT = 1
STATUS_BARRIER_TIMEOUT = 2
HOLE_SCRATCH_HEADER = 8
ISB_SKIP_FINE_GUIDE = 1
PIXEL_U8 = 0
PIXEL_F32 = 1
SSG_EVAL_MAX_THRESHOLDS = 16
SSG_EVAL_FIXED_METRICS = 4


class NativeLibraryError(RuntimeError):
    """The CUDA library is not built or cannot be loaded."""


class SSGError(RuntimeError):
    """A library call failed on the device side (``code``: the SSG_ERR_* status)."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


class ssg_camera(ctypes.Structure):
    _fields_ = [("fx", ctypes.c_float), ("fy", ctypes.c_float), ("cx", ctypes.c_float), ("cy", ctypes.c_float),
                ("xi", ctypes.c_double), ("alpha", ctypes.c_double)]


class ssg_intrinsics(ctypes.Structure):
    _fields_ = [("fx", ctypes.c_float), ("fy", ctypes.c_float), ("cx", ctypes.c_float), ("cy", ctypes.c_float),
                ("xi", ctypes.c_float), ("alpha", ctypes.c_float)]


class ssg_uneven_instance(ctypes.Structure):
    _fields_ = [("cols", ctypes.c_int), ("rows", ctypes.c_int), ("camera_count", ctypes.c_int),
                ("reference_camera", ctypes.c_int), ("candidate_count", ctypes.c_int),
                ("cameras", ctypes.c_void_p), ("relative_poses", ctypes.c_void_p), ("candidates", ctypes.c_void_p),
                ("sigma_i", ctypes.c_double), ("sigma_s", ctypes.c_double),
                ("d_staged", ctypes.c_void_p), ("d_images", ctypes.c_void_p), ("d_plane_flags", ctypes.c_void_p),
                ("d_selected", ctypes.c_void_p), ("d_guides", ctypes.c_void_p),
                ("d_costs", ctypes.c_void_p), ("d_df_guides", ctypes.c_void_p), ("d_df_costs", ctypes.c_void_p),
                ("d_distance_raw", ctypes.c_void_p), ("d_distance", ctypes.c_void_p), ("d_index", ctypes.c_void_p)]


class ssg_uneven_job(ctypes.Structure):
    _fields_ = [("cols", ctypes.c_int), ("rows", ctypes.c_int), ("references", ctypes.c_int),
                ("pano_cols", ctypes.c_int), ("pano_rows", ctypes.c_int), ("image_cols", ctypes.c_int),
                ("image_rows", ctypes.c_int), ("intrinsics", ctypes.c_void_p), ("translations", ctypes.c_void_p),
                ("d_distance", ctypes.c_void_p), ("d_tables", ctypes.c_void_p), ("d_lut", ctypes.c_void_p),
                ("d_weights", ctypes.c_void_p), ("d_images", ctypes.c_void_p), ("d_pano_distance", ctypes.c_void_p),
                ("d_rgb", ctypes.c_void_p)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_F = ctypes.c_float
_D = ctypes.c_double

# name -> (restype, argtypes); must match include/sphere_stereo_gb300.h
SIGNATURES = {
    "ssg_last_error": (ctypes.c_char_p, []),
    "ssg_version": (_I, []),
    "ssg_limits": (None, [_P]),
    "ssg_rgb_to_guide": (_I, [_P, _I64, _P, _P]),
    "ssg_select_camera": (_I, [_I, _I, _I, _P, _I, _P, _P, _D, _D, _P, _P]),
    "ssg_sweep_cost": (_I, [_I, _I, _I, _P, _I, _P, _P, _P, _P, _I, _P, _P]),
    "ssg_isb_downsample": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _F, _P]),
    "ssg_isb_upsample": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _F, _F, _F, _P]),
    "ssg_isb_level_count": (_I, [_I, _I]),
    "ssg_isb_apply": (_I, [_P, _P, _I, _I, _I, _I, _D, _D, _P]),
    "ssg_select_distance": (_I, [_P, _I, _I64, _P, _P, _P, _P]),
    "ssg_isb_upsample_select": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _F, _F, _F, _P, _P, _P, _P]),
    "ssg_inpainting_table": (_I, [_I, _I, _P, _P, _D, _D, _P, _P]),
    "ssg_box_filter": (_I, [_P, _I, _I, _I, _I, _F, _P, _P]),
    "ssg_blending_lut": (_I, [_I, _I, _I, _I, _I, _P, _P, _P, _P, _D, _D, _P, _P, _P]),
    "ssg_normalize_weights": (_I, [_P, _I, _I64, _P]),
    "ssg_reproject_distance": (_I, [_P, _P, _I, _I, _P, _P, _I, _P]),
    "ssg_inpaint": (_I, [_P, _P, _P, _I, _I, _D, _I, _P]),
    "ssg_merge_panorama": (_I, [_P, _P, _P, _P, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I, _P, _P, _P]),
    "ssg_stage_images": (_I, [_P, _I, _I, _I, _I, _P, _I, _P, _P, _P, _P]),
    "ssg_stage_images_u8": (_I, [_P, _I, _I, _I, _I, _P, _I, _P, _P, _P, _P]),
    "ssg_sweep_cost_batch": (_I, [_I, _I, _I, _I, _P, _I, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P, _P]),
    "ssg_isb_filter_batch": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _P, _P, _F, _P]),
    "ssg_stage_images_resized": (_I, [_P, _I, _I, _I, _I, _I, _I, _P, _I, _P, _P, _P, _P]),
    "ssg_sweep_cost_batch_entries": (_I, [_I, _I, _I, _I, _P, _I, _P, _P, _P, _I, _P, _P, _P, _P, _I, _I, _P,
                                          _P]),
    "ssg_isb_downsample_batch": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I, _F, _P]),
    "ssg_isb_upsample_batch": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I, _F, _F, _F, _P]),
    "ssg_isb_upsample_select_batch": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I, _F, _F, _F, _P, _P, _P, _P,
                                           _P]),
    "ssg_select_distance_batch": (_I, [_P, _I, _I64, _I, _I, _P, _P, _P, _P]),
    "ssg_isb_apply_batch": (_I, [_P, _P, _I, _I, _I, _I, _I, _D, _D, _I, _P]),
    "ssg_reproject_distance_batch": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _I, _P]),
    "ssg_reproject_distance_batch_approx": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _I, _P]),
    "ssg_inpaint_batch": (_I, [_P, _P, _P, _I, _I, _I, _I, _D, _I, _P]),
    "ssg_inpaint_holes_batch": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _D, _I, _P]),
    "ssg_inpaint_noalloc": (_I, [_P, _P, _I, _I, _D, _I, _P]),
    "ssg_isb_upsample_softargmin": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _F, _F, _F, _P, _F, _P, _P]),
    "ssg_isb_upsample_softargmin_backward": (_I, [_P, _P, _I, _I, _P, _P, _I, _I, _I, _F, _F, _F, _P, _F, _P, _P,
                                                  _P]),
    "ssg_isb_upsample_transpose": (_I, [_P, _I, _I, _P, _I, _I, _I, _F, _F, _F, _P, _P, _P, _P]),
    "ssg_isb_downsample_transpose": (_I, [_P, _I, _I, _I, _I, _I, _F, _P, _P, _P]),
    "ssg_sweep_backward_scratch_bytes": (ctypes.c_size_t, [_I, _I, _I]),
    "ssg_sweep_cost_backward": (_I, [_I, _I, _I, _P, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P, _P]),
    "ssg_merge_panorama_batch": (_I, [_P, _P, _P, _P, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P, _P]),
    "ssg_convert_u8": (_I, [_P, _P, _I64, _P]),
    "ssg_tuning_set": (_I, [_I, _I]),
    "ssg_tuning_get": (_I, [_I]),
    "ssg_tuning_choices": (_I, [_I, _P, _I]),
    "ssg_take_device_status": (_I, [_P]),
    "ssg_uneven_create": (_I, [_P, _I, _P, _I, _I, _D, _I, _P, _P, _P]),
    "ssg_uneven_upload": (_I, [_P, _P, _P, _P]),
    "ssg_uneven_run": (_I, [_P, _P]),
    "ssg_uneven_launches": (_I, [_P]),
    "ssg_uneven_destroy": (None, [_P]),
    "ssg_merge_panorama_batch_approx": (_I, [_P, _P, _P, _P, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P, _P]),
    "ssg_merge_panorama_batch_approx_images": (_I, [_P, _P, _P, _P, _P, _I, _P, _I, _I, _P, _P, _I, _I, _I, _I, _I,
                                                    _I, _P, _P, _P]),
    "ssg_resize_linear": (_I, [_P, _I, _I, _I, _I, _P, _I, _I, _I, _I, _P]),
    "ssg_eval_scratch_bytes": (ctypes.c_size_t, [_I, _I]),
    "ssg_eval_panoramas": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P]),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def library() -> ctypes.CDLL:
    """Load (once) and return the library; raises NativeLibraryError when it is unavailable."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIBRARY):
            raise NativeLibraryError(
                f"{LIBRARY} is not built; run `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(needs nvcc) -- there is no CPU fallback")
        try:
            lib = ctypes.CDLL(LIBRARY)
        except OSError as e:
            raise NativeLibraryError(f"cannot load {LIBRARY}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    return library().ssg_last_error().decode(errors="replace")


def check(code: int, what: str) -> None:
    if code == SSG_OK:
        return
    msg = f"{what}: {last_error()}"
    if code == SSG_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise SSGError(msg, code)


def call(name: str, *args) -> None:
    check(getattr(library(), name)(*args), name)


def stream_of(t: torch.Tensor) -> int:
    if t.device.type != "cuda":
        raise ValueError(f"expected a CUDA tensor, got one on {t.device}")
    return torch.cuda.current_stream(t.device).cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def require(t: torch.Tensor, name: str, dtype: torch.dtype, shape: tuple | None = None, device=None) -> None:
    """Argument validation before any launch (the reference has none; see the module docstring
    of depth_estimation.py)."""
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if t.device.type != "cuda":
        raise ValueError(f"{name} must be a CUDA tensor (got {t.device}); there is no CPU path")
    if device is not None and t.device != torch.device(device):
        raise ValueError(f"{name} is on {t.device}, expected {device}")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype} (got {t.dtype})")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)} (got {tuple(t.shape)})")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def cameras_array(cams: list[ssg_camera]):
    return (ssg_camera * len(cams))(*cams)


def intrinsics_array(ks: list[ssg_intrinsics]):
    return (ssg_intrinsics * len(ks))(*ks)


def floats(values) -> ctypes.Array:
    values = [float(v) for v in values]
    return (ctypes.c_float * len(values))(*values)


def ints(values) -> ctypes.Array:
    values = [int(v) for v in values]
    return (ctypes.c_int * len(values))(*values)


def pointers(values) -> ctypes.Array:
    return (ctypes.c_void_p * len(values))(*[int(v) for v in values])


def hole_filling_launches(iterations: int) -> int:
    """Kernels one batched hole filling of a uniform batch launches: the scan and step 1, then one
    cooperative launch for the other steps (SSG_TUNE_HOLE_PERSISTENT), or a launch per step up to
    the tail (SSG_TUNE_HOLE_TAIL) and two for the tail."""
    if iterations <= 1:
        return 2 * iterations
    lib = library()
    if lib.ssg_tuning_get(TUNE_HOLE_PERSISTENT) == 1:
        return 3
    tail = lib.ssg_tuning_get(TUNE_HOLE_TAIL)
    if tail > 0 and iterations >= tail:
        return tail + 2
    return 1 + iterations


def isb_tail_first(rows: int, cols: int, levels: int, max_pixels: int) -> int:
    """The first level of a pyramid's fused tail (the library's rule): the first level s >= 1 of at
    most max_pixels pixels with s <= levels - 2, else levels (no tail)."""
    if max_pixels <= 0:
        return levels
    for s in range(1, levels - 1):
        if math.ceil(rows / 2 ** s) * math.ceil(cols / 2 ** s) <= max_pixels:
            return s
    return levels


def isb_filter_launches(rows: int, cols: int, levels: int) -> int:
    """Kernels ssg_isb_filter_batch launches: a down step per level up to the tail's first, the
    tail, an up step per level below it (SSG_TUNE_ISB_TAIL)."""
    first = isb_tail_first(rows, cols, levels, library().ssg_tuning_get(TUNE_ISB_TAIL))
    return 2 * first if first < levels else (levels - 1) + (levels - 2)


def isb_apply_launches(rows: int, cols: int, levels: int, candidates: int) -> int:
    """Kernels ssg_isb_apply_batch launches (the single-candidate filter fuses its small levels,
    SSG_TUNE_POST_TAIL)."""
    first = isb_tail_first(rows, cols, levels, library().ssg_tuning_get(TUNE_POST_TAIL)) if candidates == 1 \
        else levels
    return 2 * first + 1 if first < levels else 2 * max(0, levels - 1)


def kernels_launched(name: str, args) -> int:
    """Number of kernels one call of entry point ``name`` with ``args`` launches."""
    if name in ("ssg_last_error", "ssg_version", "ssg_limits", "ssg_isb_level_count", "ssg_tuning_set",
                "ssg_tuning_get", "ssg_tuning_choices", "ssg_eval_scratch_bytes", "ssg_take_device_status"):
        return 0
    if name == "ssg_eval_panoramas":
        return 3
    if name == "ssg_isb_apply":
        return 2 * max(0, int(args[2]) - 1)
    if name == "ssg_isb_apply_batch":
        return isb_apply_launches(int(args[3]), int(args[4]), int(args[2]), int(args[5]))
    if name == "ssg_isb_filter_batch":
        return isb_filter_launches(int(args[3]), int(args[4]), int(args[2]))
    if name == "ssg_reproject_distance":
        return 2 if args[6] else 1
    if name in ("ssg_reproject_distance_batch", "ssg_reproject_distance_batch_approx"):
        return 2 if args[8] else 1
    if name == "ssg_inpaint":
        return -(-int(args[6]) // 16)
    if name == "ssg_inpaint_holes_batch":
        return hole_filling_launches(int(args[9]))
    if name == "ssg_inpaint_batch":
        return -(-int(args[8]) // 16)
    if name == "ssg_inpaint_noalloc":
        return -(-int(args[5]) // 16)
    return 1

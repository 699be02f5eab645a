"""The C ABI surface, without a GPU: the library loads, exports every function that
include/sphere_stereo_gb300.h declares, the ctypes binding agrees with the header, and invalid
arguments are rejected with an error code and a message before anything touches a device."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "sphere_stereo_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"SSG_API\s+([\w\s\*]+?)\b(ssg_\w+)\s*\(([^)]*)\)\s*;", text):
        args = [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(2)] = args
    return out


def test_header_declares_the_abi():
    decl = declared()
    assert len(decl) >= 19
    for name in ("ssg_sweep_cost", "ssg_isb_apply", "ssg_isb_upsample_select", "ssg_inpaint", "ssg_merge_panorama"):
        assert name in decl


def test_library_exports_every_declared_symbol(native):
    for name in declared():
        assert hasattr(native, name), name


def test_binding_matches_header(ss):
    decl = declared()
    sigs = ss._native.SIGNATURES
    assert set(sigs) == set(decl)
    for name, args in decl.items():
        assert len(sigs[name][1]) == len(args), name


def test_version_and_limits(native, ss):
    assert native.ssg_version() >= 100
    out = (ctypes.c_int32 * 4)()
    native.ssg_limits(out)
    assert list(out) == [ss._native.MAX_CAMERAS, ss._native.MAX_CANDIDATES, ss._native.MAX_REFERENCES,
                         ss._native.MAX_LEVELS]


def test_invalid_arguments_rejected_without_a_device(native, ss):
    N = ss._native
    assert native.ssg_rgb_to_guide(None, 10, None, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "null" in N.last_error()
    assert native.ssg_select_distance(None, 4, 10, None, None, None, None) == N.SSG_ERR_INVALID_ARGUMENT
    # a 2x downsampling must halve the size
    assert native.ssg_isb_downsample(1, 1, 10, 10, 1, 1, 8, 5, 3, 0.1, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "downsampling" in N.last_error()
    # pyramid depth must match the image
    ptrs = N.pointers([1] * 3)
    assert native.ssg_isb_apply(ptrs, ptrs, 3, 64, 64, 4, 10.0, 25.0, None) == N.SSG_ERR_INVALID_ARGUMENT
    cams = N.cameras_array([N.ssg_camera(100, 100, 32, 32, -0.2, 0.6)] * 2)
    poses = N.floats([0.0] * 24)
    assert native.ssg_sweep_cost(64, 64, 2, cams, 0, poses, N.pointers([1, 1]), 1, N.floats([1.0] * 3), 300, 1,
                                 None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "candidate_count" in N.last_error()
    bad = N.cameras_array([N.ssg_camera(100, 100, 32, 32, -0.2, 1.5)] * 2)
    assert native.ssg_sweep_cost(64, 64, 2, bad, 0, poses, N.pointers([1, 1]), 1, N.floats([1.0] * 3), 3, 1,
                                 None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "alpha" in N.last_error()
    with pytest.raises(ValueError):
        N.call("ssg_rgb_to_guide", None, 10, None, None)


def test_misaligned_cells_and_entries_rejected_without_a_device(native, ss):
    """32-byte units (float32 cost cells, the fixed-point footprint entries of float inputs) move
    as single 256-bit accesses: every entry point refuses a buffer that is not 32-byte aligned
    (16 bytes for 16-bit cells) before anything is launched."""
    N = ss._native
    A, M = 0x100000, 0x100010  # 32-byte aligned / 16-byte but not 32-byte aligned
    F16, F32 = 0, 2
    # downsampling: float32 input cells, then float32 output cells
    assert native.ssg_isb_downsample_batch(A, M, 64, 64, A, A, 32, 32, 32, 1, F32, 0.1, None) == \
        N.SSG_ERR_INVALID_ARGUMENT
    assert "d_cost_in must be 32-byte aligned" in N.last_error()
    assert native.ssg_isb_downsample_batch(A, M, 64, 64, A, M, 32, 32, 32, 1, F16, 0.1, None) == \
        N.SSG_ERR_INVALID_ARGUMENT
    assert "d_cost_out must be 32-byte aligned" in N.last_error()
    assert native.ssg_isb_downsample_batch(A, A + 8, 64, 64, A, A, 32, 32, 32, 1, F16, 0.1, None) == \
        N.SSG_ERR_INVALID_ARGUMENT
    assert "16-byte aligned" in N.last_error()
    # coarse upsampling: the fine float32 cells are read and written whole
    assert native.ssg_isb_upsample_batch(A, A, 32, 32, A, M, 64, 64, 32, 1, F32, 0.5, 0.5, 0.1, None) == \
        N.SSG_ERR_INVALID_ARGUMENT
    assert "d_cost_inout must be 32-byte aligned" in N.last_error()
    cand = N.floats([1.0 + k for k in range(32)])
    assert native.ssg_isb_upsample_select_batch(A, A, 32, 32, A, M, 64, 64, 32, 1, F32, 0.5, 0.5, 0.1, cand, A, A,
                                                None, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "d_cost_fine must be 32-byte aligned" in N.last_error()
    assert native.ssg_select_distance_batch(M, 32, 64 * 64, 1, F32, cand, A, A, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "d_cost must be 32-byte aligned" in N.last_error()
    # staging and sweep of float images: 32-byte footprint entries
    refs = N.ints([0])
    assert native.ssg_stage_images(A, 1, 2, 64, 64, refs, 1, M, A, A, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "32-byte aligned" in N.last_error()
    cams = N.cameras_array([N.ssg_camera(100, 100, 32, 32, -0.2, 0.6)] * 2)
    poses = N.floats([0.0] * 24)
    assert native.ssg_sweep_cost_batch(64, 64, 1, 2, cams, 1, refs, poses, M, A, A, A, cand, 32, F16, A, None) == \
        N.SSG_ERR_INVALID_ARGUMENT
    assert "32-byte aligned" in N.last_error()


def test_resized_staging_and_entry_sizes_checked_without_a_device(native, ss):
    """The one-pass resize + staging refuses misaligned planes, and declines (SSG_ERR_UNSUPPORTED,
    so that the caller resizes first) sources whose images do not start on 4-byte boundaries or
    whose tile windows would not fit in shared memory; the sweep's entry size is 16 or 32 bytes,
    32 whenever float images are given.  All before anything is launched."""
    N = ss._native
    A, M = 0x100000, 0x100010
    refs = N.ints([0])
    assert native.ssg_stage_images_resized(A, 1216, 1216, 1, 2, 1024, 1024, refs, 1, M, A, A, None) == \
        N.SSG_ERR_INVALID_ARGUMENT
    assert "32-byte" in N.last_error()
    assert native.ssg_stage_images_resized(A, 33, 35, 1, 2, 20, 20, refs, 1, A, A, A, None) == N.SSG_ERR_UNSUPPORTED
    assert "4-byte" in N.last_error()
    assert native.ssg_stage_images_resized(A + 2, 64, 64, 1, 2, 20, 20, refs, 1, A, A, A, None) == \
        N.SSG_ERR_UNSUPPORTED
    # the shared-memory tile staging declines windows beyond its limit (the column staging has none)
    saved = native.ssg_tuning_get(N.TUNE_STAGE_COLUMNS)
    assert native.ssg_tuning_set(N.TUNE_STAGE_COLUMNS, 0) == 0
    try:
        assert native.ssg_stage_images_resized(A, 4096, 4096, 1, 2, 256, 256, refs, 1, A, A, A, None) == \
            N.SSG_ERR_UNSUPPORTED
        assert "shared memory" in N.last_error()
    finally:
        native.ssg_tuning_set(N.TUNE_STAGE_COLUMNS, saved)
    cams = N.cameras_array([N.ssg_camera(100, 100, 32, 32, -0.2, 0.6)] * 2)
    poses = N.floats([0.0] * 24)
    cand = N.floats([1.0 + k for k in range(32)])
    assert native.ssg_sweep_cost_batch_entries(64, 64, 1, 2, cams, 1, refs, poses, A, 24, None, A, A, cand, 32, 0,
                                               A, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "entry_bytes" in N.last_error()
    assert native.ssg_sweep_cost_batch_entries(64, 64, 1, 2, cams, 1, refs, poses, A, 16, A, A, A, cand, 32, 0,
                                               A, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert native.ssg_sweep_cost_batch_entries(64, 64, 1, 2, cams, 1, refs, poses, M, 32, None, A, A, cand, 32, 0,
                                               A, None) == N.SSG_ERR_INVALID_ARGUMENT
    assert "32-byte aligned" in N.last_error()

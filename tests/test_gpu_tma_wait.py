"""The bounded wait of the TMA-staged ISB upsampling, made to run out on purpose.

SSG_TUNE_TMA_WITHHOLD = 1 makes every block arm its tile barrier without issuing the copy, so its
first wait runs out after a short limit: a flag that nothing sets.  No copy is in flight, nothing
faults.  The launch must return, report SSG_STATUS_TMA_TIMEOUT through ssg_take_device_status, and
write no candidate cell and no selection; the next normal launch must be clean and give the
cp.async staging's bits."""
from __future__ import annotations

import ctypes
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _status(N) -> int:
    s = ctypes.c_uint32(0)
    N.call("ssg_take_device_status", ctypes.byref(s))
    return int(s.value)


def _case(seed=5, rows_f=96, cols_f=150, n=16, inst=2):
    rng = np.random.default_rng(seed)
    rows_c, cols_c = (rows_f + 1) // 2, (cols_f + 1) // 2
    chunks = (n + 7) // 8
    guide_c = rng.integers(16, 236, (inst, rows_c, cols_c, 4), dtype=np.uint8)
    guide_f = rng.integers(16, 236, (inst, rows_f, cols_f, 4), dtype=np.uint8)
    guide_c[..., 3] = 0
    guide_f[..., 3] = 0
    cost_c = (rng.random((inst, chunks, rows_c * cols_c, 8)) * 400).astype(np.float32)
    cost_f = (rng.random((inst, chunks, rows_f * cols_f, 8)) * 400).astype(np.float16)
    return dict(rows_c=rows_c, cols_c=cols_c, rows_f=rows_f, cols_f=cols_f, n=n, inst=inst, guide_c=guide_c,
                guide_f=guide_f, cost_c=cost_c, cost_f=cost_f)


def _select(N, c, candidates):
    """ssg_isb_upsample_select_batch on fresh copies; outputs pre-filled with a NaN pattern."""
    t = {k: torch.as_tensor(c[k].copy(), device=DEV) for k in ("guide_c", "guide_f", "cost_c")}
    cost_f = torch.as_tensor(c["cost_f"].view(np.int16).copy(), device=DEV)
    pixels = c["inst"] * c["rows_f"] * c["cols_f"]
    dist = torch.full((pixels,), float("nan"), device=DEV)
    index = torch.full((pixels,), -7, dtype=torch.int32, device=DEV)
    N.call("ssg_isb_upsample_select_batch", t["guide_c"].data_ptr(), t["cost_c"].data_ptr(), c["rows_c"],
           c["cols_c"], t["guide_f"].data_ptr(), cost_f.data_ptr(), c["rows_f"], c["cols_f"], c["n"], c["inst"], 0,
           0.8, 0.3, 1 / 200, candidates, dist.data_ptr(), index.data_ptr(), None,
           torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return dist.cpu().numpy(), index.cpu().numpy()


def _upsample(N, c):
    """ssg_isb_upsample_batch (float32 fine level, filtered in place) on fresh copies."""
    t = {k: torch.as_tensor(c[k].copy(), device=DEV) for k in ("guide_c", "guide_f", "cost_c")}
    fine = torch.as_tensor(c["cost_f"].astype(np.float32), device=DEV)
    N.call("ssg_isb_upsample_batch", t["guide_c"].data_ptr(), t["cost_c"].data_ptr(), c["rows_c"], c["cols_c"],
           t["guide_f"].data_ptr(), fine.data_ptr(), c["rows_f"], c["cols_f"], c["n"], c["inst"], 2, 0.8, 0.3,
           1 / 200, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return fine.cpu().numpy()


def test_tma_wait_runs_out_reports_and_writes_nothing(ss, native):
    N = ss._native
    tune = importlib.import_module("sphere-stereo_gb300.autotune")
    c = _case()
    candidates = N.floats(1 / np.linspace(1 / 0.55, 1 / 100.0, c["n"]))
    saved = tune.get("isb_tile_tma")
    _status(N)  # start from a clear word
    try:
        tune.set_knob("isb_tile_tma", 0)
        want_d, want_i = _select(N, c, candidates)
        want_up = _upsample(N, c)
        assert _status(N) == 0
        tune.set_knob("isb_tile_tma", 1)
        N.call("ssg_tuning_set", N.TUNE_TMA_WITHHOLD, 1)
        try:
            d, i = _select(N, c, candidates)
            assert _status(N) == N.STATUS_TMA_TIMEOUT
            assert np.isnan(d).all() and (i == -7).all(), "a block whose tile never landed wrote a selection"
            up = _upsample(N, c)
            assert _status(N) == N.STATUS_TMA_TIMEOUT
            # the first chunk's tile never lands: no candidate cell is written
            np.testing.assert_array_equal(up, c["cost_f"].astype(np.float32))
        finally:
            N.call("ssg_tuning_set", N.TUNE_TMA_WITHHOLD, 0)
        # the word was cleared by the read; the next launches are clean and exact
        d, i = _select(N, c, candidates)
        up = _upsample(N, c)
        assert _status(N) == 0
        np.testing.assert_array_equal(d, want_d)
        np.testing.assert_array_equal(i, want_i)
        np.testing.assert_array_equal(up, want_up)
    finally:
        tune.set_knob("isb_tile_tma", saved)


def test_pipeline_falls_back_when_a_tma_wait_runs_out(ss, native, golden_small):
    """A batch run with TMA staging whose wait runs out is detected by the pipeline, which warns,
    switches the knob back to cp.async and runs the batch again: the results are the cp.async
    ones."""
    N = ss._native
    tune = importlib.import_module("sphere-stereo_gb300.autotune")
    from test_gpu_batch import _batch, _estimator

    g = golden_small
    saved = tune.get("isb_tile_tma")
    _status(N)
    try:
        tune.set_knob("isb_tile_tma", 0)
        est, _ = _estimator(ss, g, "fp16", max_batch=1, graphs=False)
        match, stitch = _batch(g)
        rgb0, d0 = (t.clone() for t in est.estimate_RGBD_panoramas(match, stitch))
        tune.set_knob("isb_tile_tma", 1)
        N.call("ssg_tuning_set", N.TUNE_TMA_WITHHOLD, 1)
        try:
            with pytest.warns(RuntimeWarning, match="TMA"):
                rgb1, d1 = est.estimate_RGBD_panoramas(match, stitch)
        finally:
            N.call("ssg_tuning_set", N.TUNE_TMA_WITHHOLD, 0)
        assert tune.get("isb_tile_tma") == 0
        torch.testing.assert_close(rgb1, rgb0, rtol=0, atol=0)
        torch.testing.assert_close(d1, d0, rtol=0, atol=0)
        assert _status(N) == 0
    finally:
        tune.set_knob("isb_tile_tma", saved)

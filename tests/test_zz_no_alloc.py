"""ssg_inpaint_noalloc, the hole-filling entry point for callers that cannot allocate device
memory (for instance a plugin whose host application's memory manager owns the device heap, or
a real-time loop that must not risk cudaMalloc's synchronisation).  Its scratch map is a fixed
array inside the library; the caller passes only the map and the table.

Checked through the C ABI against ssg_inpaint (which takes a caller-allocated scratch map) on
two calls in a row, with different maps, so that what the first call leaves in the shared
array cannot leak into the second.  This file is collected last; it needs nothing from the other
tests and passes in a fresh process on its own."""
from __future__ import annotations

import numpy as np
import pytest
import torch

DEV = "cuda:0"
MAX_PIXELS = 1 << 20


def _case(seed, rows, cols):
    rng = np.random.default_rng(seed)
    d = (1 + rng.random((rows, cols)) * 9).astype(np.float32)
    d[rows // 5: rows // 2, cols // 4: cols // 2] = 1e8
    d[rng.random((rows, cols)) < 0.15] = 1e8
    table = rng.integers(0, 256, (rows, cols, 2)).astype(np.uint8)
    return torch.as_tensor(d, device=DEV), torch.as_tensor(table, device=DEV)


def _with_scratch(ss, d, table, iterations):
    out = d.clone()
    scratch = torch.empty_like(d)
    rows, cols = d.shape
    ss._native.call("ssg_inpaint", out.data_ptr(), table.data_ptr(), scratch.data_ptr(), cols, rows, 100.0, iterations,
                    torch.cuda.current_stream().cuda_stream)
    return out


def _no_alloc(ss, d, table, iterations):
    out = d.clone()
    rows, cols = d.shape
    ss._native.call("ssg_inpaint_noalloc", out.data_ptr(), table.data_ptr(), cols, rows, 100.0, iterations,
                    torch.cuda.current_stream().cuda_stream)
    return out


@pytest.mark.gpu
def test_no_alloc_inpaint_matches_allocating_entry_point(ss, native):
    # two calls in a row on different maps: a full-size 1024 x 1024 map with the reference's 32
    # iterations (two passes), then a smaller odd-sized one with an odd iteration count
    for seed, (rows, cols), iterations in ((1, (1024, 1024), 32), (2, (333, 517), 17)):
        d, table = _case(seed, rows, cols)
        want = _with_scratch(ss, d, table, iterations)
        got = _no_alloc(ss, d, table, iterations)
        torch.cuda.synchronize()
        # both run the same Jacobi steps on the same tiles: identical to the bit
        torch.testing.assert_close(got, want, rtol=0, atol=0)
        assert (got.cpu().numpy() < 1e8).mean() > (d.cpu().numpy() < 1e8).mean()  # holes were filled


@pytest.mark.gpu
def test_no_alloc_inpaint_rejects_maps_beyond_its_scratch(ss, native):
    d = torch.zeros(1, device=DEV)
    code = native.ssg_inpaint_noalloc(d.data_ptr(), d.data_ptr(), 1025, 1024, 100.0, 32, None)
    assert code == ss._native.SSG_ERR_UNSUPPORTED
    assert "1049600 pixels" in ss._native.last_error()
    assert MAX_PIXELS == 1024 * 1024

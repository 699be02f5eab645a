"""ISB_Filter: the reference's edge-preserving multiscale filter (python/isb_filter.py:35-136),
same constructor and ``apply`` contract, running the sm_103a kernels of csrc/ssg_isb.cu."""
from __future__ import annotations

import math

import torch

from . import _native as N


def level_shapes(resolution) -> list[tuple[int, int]]:
    """(rows, cols) of every pyramid level: int(min(log2 cols, log2 rows) - 1) levels of
    ceil(dim / 2^s) (python/isb_filter.py:58-70)."""
    cols, rows = resolution
    count = int(min(math.log2(cols), math.log2(rows)) - 1)
    return [(math.ceil(rows / (2 ** s)), math.ceil(cols / (2 ** s))) for s in range(count)]


def level_weights(scale_count: int, sigma_s: float) -> list[tuple[float, float]]:
    """(weight_up, weight_down) of each upsampling step s (python/isb_filter.py:110-112)."""
    var_inv_s = 1 / (2 * sigma_s * sigma_s)
    out = []
    for scale in range(scale_count - 1):
        distance = 2 ** scale - 0.5
        weight_down = math.exp(-(distance * distance) * var_inv_s)
        out.append((1 - weight_down, weight_down))
    return out


class ISB_Filter:
    def __init__(self, candidate_count, resolution, device):
        """Fast edge-preserving filter; allocates the intermediate scales.

        Args:
            candidate_count: number of channels of the quantity to filter (distance candidates
                for cost volumes)
            resolution: (cols, rows) of the guide and cost
            device: the CUDA device that holds the guide and cost
        """
        device = torch.device(device)
        if device.type != "cuda":
            raise ValueError(f"ISB_Filter runs on a CUDA device, got {device}; there is no CPU path")
        self.candidate_count = candidate_count
        self.resolution = tuple(resolution)
        self.device = device
        shapes = level_shapes(resolution)
        self.scale_count = len(shapes)
        self.guides = [torch.zeros([r, c, 3], dtype=torch.uint8, device=device) for r, c in shapes]
        self.costs = [torch.zeros([candidate_count, r, c], device=device) for r, c in shapes]
        N.library()

    def apply(self, guide, cost, sigma_i, sigma_s):
        """Filter ``cost`` guided by ``guide``, both in place (python/isb_filter.py:72-136).

        Args:
            guide: [rows, cols, 3] uint8 guide (YCbCr works best)
            cost: [candidate_count, rows, cols] float32 quantity to smooth
            sigma_i: edge preservation; lower values preserve edges more
            sigma_s: smoothing; higher values give coarser scales more weight
        Returns:
            cost, guide: the filtered cost volume and guide (the tensors passed in)
        """
        cols, rows = self.resolution
        N.require(guide, "guide", torch.uint8, (rows, cols, 3), self.device)
        N.require(cost, "cost", torch.float32, (self.candidate_count, rows, cols), self.device)
        self.guides[0] = guide
        self.costs[0] = cost
        if self.scale_count < 2:
            return self.costs[0], self.guides[0]
        N.call("ssg_isb_apply", N.pointers([g.data_ptr() for g in self.guides]),
               N.pointers([c.data_ptr() for c in self.costs]), self.scale_count, rows, cols, self.candidate_count,
               float(sigma_i), float(sigma_s), N.stream_of(cost))
        return self.costs[0], self.guides[0]

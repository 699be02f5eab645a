"""Differentiable sphere sweep for calibration refinement (no counterpart in the reference, which
selects distances with a hard argmin, python/depth_estimation.py:179-198).

``DifferentiableSweep(...)(images, pose_deltas)`` returns, for every reference camera, the
soft-argmin inverse distance

    q = sum_k softmax(-F_k / temperature) / d_k ,

F being the ISB-filtered sweep cost (python/depth_estimation.py:141-177, the fp32 kernels of the
library).  It is differentiable with respect to the matching images and to per-camera 6-DoF
pose deltas delta_c = (omega_c, v_c), the camera poses being T_c [Exp(omega_c), v_c].  The
backward pass recomputes the cost volume and the filter pyramid instead of storing them, runs
the filter transposed (its weights come from uint8 guides and get no gradient), and reduces the
pose gradient per camera in float64; the pose composition is float64 on the host.  The gradients
are bit-reproducible run to run: the transposed filter steps gather in a fixed order, the image
gradient is summed in 64-bit fixed point and the pose gradient by a fixed float64 tree.

Temperature: 2 cost units by default.  Costs are sums of three absolute 8-bit differences; near
the minimum, neighbouring candidates typically differ by a few units, so tau = 2 keeps the
weights concentrated on the best few candidates while staying smooth.
"""
from __future__ import annotations

import math

import torch

from . import _native as N
from .isb_filter import level_shapes, level_weights
from .utils import _cpu32, camera_struct, relative_poses, rgb_to_guide


def skew(w):
    return torch.tensor([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]], dtype=torch.float64)


def so3_exp(w: torch.Tensor) -> torch.Tensor:
    th = float(torch.linalg.norm(w))
    k = skew(w)
    if th < 1e-8:
        return torch.eye(3, dtype=torch.float64) + k + 0.5 * k @ k
    return torch.eye(3, dtype=torch.float64) + math.sin(th) / th * k + (1 - math.cos(th)) / th ** 2 * k @ k


def so3_right_jacobian(w: torch.Tensor) -> torch.Tensor:
    th = float(torch.linalg.norm(w))
    k = skew(w)
    if th < 1e-6:
        return torch.eye(3, dtype=torch.float64) - 0.5 * k + k @ k / 6
    return (torch.eye(3, dtype=torch.float64) - (1 - math.cos(th)) / th ** 2 * k
            + (th - math.sin(th)) / th ** 3 * k @ k)


class DifferentiableSweep:
    def __init__(self, calibrations, min_dist, max_dist, candidate_count, references_indices, masks,
                 matching_resolution, sigma_i, sigma_s, device, temperature: float = 2.0):
        """Same camera, range and filter arguments as RGBD_Estimator (python/depth_estimation.py:39-40)."""
        device = torch.device(device)
        if device.type != "cuda":
            raise ValueError(f"DifferentiableSweep runs on a CUDA device, got {device}; there is no CPU path")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        N.library()
        if temperature <= 0:
            raise ValueError("temperature must be positive")
        self.device = device
        self.calibrations = calibrations
        self.C = len(calibrations)
        self.refs = list(references_indices)
        self.cols, self.rows = matching_resolution
        self.P = self.cols * self.rows
        self.N = candidate_count
        self.sigma_i, self.sigma_s = float(sigma_i), float(sigma_s)
        self.temperature = float(temperature)
        self.shapes = level_shapes(matching_resolution)
        self.L = len(self.shapes)
        if self.L < 2:
            raise ValueError("the matching resolution is too small for the filter pyramid")
        self.candidates = (1 / torch.linspace(1 / min_dist, 1 / max_dist, candidate_count)).tolist()
        self._cand = N.floats(self.candidates)
        self._cams = N.cameras_array([camera_struct(c) for c in calibrations])
        self.base_poses = [_cpu32(c.rt).double() for c in calibrations]
        dev = device
        # camera selection of the unperturbed rig (a discrete choice: no gradient)
        mask_stack = torch.stack([torch.as_tensor(m, dtype=torch.float32).reshape(self.rows, self.cols)
                                  for m in masks]).to(dev).contiguous()
        self.selected = []
        for r in self.refs:
            sel = torch.empty([self.rows, self.cols], dtype=torch.int8, device=dev)
            N.call("ssg_select_camera", self.cols, self.rows, self.C, self._cams, r,
                   N.floats(relative_poses(calibrations, r)), mask_stack.data_ptr(), float(min_dist),
                   float(max_dist), sel.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
            self.selected.append(sel)
        f32 = dict(dtype=torch.float32, device=dev)
        u8 = dict(dtype=torch.uint8, device=dev)
        self.costs = [torch.empty(self.N * r * c, **f32) for r, c in self.shapes]
        self.g_orig = [torch.empty(r * c * 3, **u8) for r, c in self.shapes]
        self.g_filt = [torch.empty(r * c * 3, **u8) for r, c in self.shapes]
        self.gf = [torch.empty(self.N * r * c, **f32) for r, c in self.shapes]
        self.gc = [torch.empty(self.N * r * c, **f32) for r, c in self.shapes]
        self.weights = level_weights(self.L, self.sigma_s)
        self.var_inv_i = 1 / (2 * self.sigma_i * self.sigma_i)
        # the sweep backward's fixed-point image sums and pose block sums
        scratch = N.library().ssg_sweep_backward_scratch_bytes(self.cols, self.rows, self.C)
        self._bwd_scratch = torch.empty((scratch + 255) // 256 * 256, dtype=torch.uint8, device=dev)

    def set_selection(self, selected):
        """Use another run's camera-selection maps ([references][rows, cols])."""
        self.selected = [torch.as_tensor(s).reshape(self.rows, self.cols).to(self.device, torch.int8).contiguous()
                         for s in selected]

    # ------------------------------------------------------------------------------------
    def _poses(self, deltas: torch.Tensor):
        """Float64 composition: T_c [Exp(omega_c), v_c] and, per reference, the relative poses."""
        d = deltas.detach().to("cpu", torch.float64)
        T = []
        for c in range(self.C):
            E = torch.eye(4, dtype=torch.float64)
            E[:3, :3] = so3_exp(d[c, :3])
            E[:3, 3] = d[c, 3:]
            T.append(self.base_poses[c] @ E)
        rel = {r: N.floats([float(v) for c in range(self.C) for v in (torch.linalg.inv(T[c]) @ T[r])[:3].reshape(12)])
               for r in self.refs}
        return d, rel

    def _pyramid(self, r: int, images: torch.Tensor, rel, stream) -> None:
        """Sweep + ISB down / up steps (levels 1..L-1 filtered; level 0 left raw)."""
        cols, rows, n = self.cols, self.rows, self.N
        rgb_to_guide(images[r], self.g_orig[0].view(rows, cols, 3))
        N.call("ssg_sweep_cost", cols, rows, self.C, self._cams, r, rel[r],
               N.pointers([images[c].data_ptr() for c in range(self.C)]), self.selected[self.refs.index(r)].data_ptr(),
               self._cand, n, self.costs[0].data_ptr(), stream)
        for s in range(1, self.L):
            (ri, ci), (ro, co) = self.shapes[s - 1], self.shapes[s]
            N.call("ssg_isb_downsample", self.g_orig[s - 1].data_ptr(), self.costs[s - 1].data_ptr(), ri, ci,
                   self.g_orig[s].data_ptr(), self.costs[s].data_ptr(), ro, co, n, self.var_inv_i, stream)
        for s in range(1, self.L):
            self.g_filt[s].copy_(self.g_orig[s])
        for s in range(self.L - 2, 0, -1):
            (rc, cc), (rf, cf) = self.shapes[s + 1], self.shapes[s]
            wu, wd = self.weights[s]
            N.call("ssg_isb_upsample", self.g_filt[s + 1].data_ptr(), self.costs[s + 1].data_ptr(), rc, cc,
                   self.g_filt[s].data_ptr(), self.costs[s].data_ptr(), rf, cf, n, wu, wd, self.var_inv_i, stream)

    def forward(self, images: torch.Tensor, deltas: torch.Tensor) -> torch.Tensor:
        N.require(images, "images", torch.float32, (self.C, self.rows, self.cols, 3), self.device)
        stream = N.stream_of(images)
        _, rel = self._poses(deltas)
        q = torch.empty(len(self.refs), self.rows, self.cols, device=self.device)
        (rc, cc) = self.shapes[1]
        wu, wd = self.weights[0]
        for slot, r in enumerate(self.refs):
            self._pyramid(r, images, rel, stream)
            N.call("ssg_isb_upsample_softargmin", self.g_filt[1].data_ptr(), self.costs[1].data_ptr(), rc, cc,
                   self.g_orig[0].data_ptr(), self.costs[0].data_ptr(), self.rows, self.cols, self.N, wu, wd,
                   self.var_inv_i, self._cand, self.temperature, q[slot].data_ptr(), stream)
        return q

    def backward(self, images: torch.Tensor, deltas: torch.Tensor, grad_q: torch.Tensor):
        stream = N.stream_of(images)
        d, rel = self._poses(deltas)
        grad_images = torch.zeros_like(images)
        grad_local = torch.zeros(self.C, 6, dtype=torch.float64, device=self.device)
        cols, rows, n = self.cols, self.rows, self.N
        for slot, r in enumerate(self.refs):
            self._pyramid(r, images, rel, stream)
            (rc, cc) = self.shapes[1]
            wu, wd = self.weights[0]
            # dL/dF of the filtered level 0, then every up step transposed from level 0 upwards:
            # each writes its level's own-pixel gradient and the next level's filtered gradient
            N.call("ssg_isb_upsample_softargmin_backward", self.g_filt[1].data_ptr(), self.costs[1].data_ptr(), rc, cc,
                   self.g_orig[0].data_ptr(), self.costs[0].data_ptr(), rows, cols, n, wu, wd, self.var_inv_i,
                   self._cand, self.temperature, grad_q[slot].data_ptr(), self.gf[0].data_ptr(), stream)
            for s in range(0, self.L - 1):
                (rc, cc), (rf, cf) = self.shapes[s + 1], self.shapes[s]
                wu, wd = self.weights[s]
                N.call("ssg_isb_upsample_transpose", self.g_filt[s + 1].data_ptr(), rc, cc, self.g_orig[s].data_ptr(),
                       rf, cf, n, wu, wd, self.var_inv_i, self.gf[s].data_ptr(), self.gc[s].data_ptr(),
                       self.gf[s + 1].data_ptr(), stream)
            self.gc[self.L - 1].copy_(self.gf[self.L - 1])  # f_{L-1} = c_{L-1}
            for s in range(self.L - 1, 0, -1):
                (ri, ci), (ro, co) = self.shapes[s - 1], self.shapes[s]
                N.call("ssg_isb_downsample_transpose", self.g_orig[s - 1].data_ptr(), ri, ci, ro, co, n,
                       self.var_inv_i, self.gc[s].data_ptr(), self.gc[s - 1].data_ptr(), stream)
            N.call("ssg_sweep_cost_backward", cols, rows, self.C, self._cams, r, rel[r],
                   N.pointers([images[c].data_ptr() for c in range(self.C)]),
                   N.pointers([grad_images[c].data_ptr() for c in range(self.C)]),
                   self.selected[slot].data_ptr(), self._cand, n, self.gc[0].data_ptr(), grad_local.data_ptr(),
                   self._bwd_scratch.data_ptr(), stream)
        # local right perturbations at T [Exp(omega), v]  ->  gradients with respect to (omega, v)
        g = grad_local.cpu()
        out = torch.empty_like(g)
        for c in range(self.C):
            w = d[c, :3]
            out[c, :3] = so3_right_jacobian(w).T @ g[c, :3]
            out[c, 3:] = so3_exp(w) @ g[c, 3:]
        return grad_images, out.to(deltas.device)

    def __call__(self, images: torch.Tensor, pose_deltas: torch.Tensor | None = None) -> torch.Tensor:
        """images [cameras, rows, cols, 3] float32; pose_deltas [cameras, 6] float64 (zeros if
        None).  Returns the soft-argmin inverse distance [references, rows, cols]."""
        if pose_deltas is None:
            pose_deltas = torch.zeros(self.C, 6, dtype=torch.float64, device=self.device)
        return _SoftSweep.apply(images, pose_deltas, self)


class _SoftSweep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, images, pose_deltas, sweep):
        images_c = images.detach().contiguous()
        ctx.save_for_backward(images_c, pose_deltas.detach())
        ctx.sweep = sweep
        return sweep.forward(images_c, pose_deltas)

    @staticmethod
    def backward(ctx, grad_q):
        images, deltas = ctx.saved_tensors
        gi, gd = ctx.sweep.backward(images, deltas, grad_q.contiguous())
        return gi, gd, None

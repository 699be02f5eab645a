"""TEST INFRASTRUCTURE -- float64 torch autograd restatement of the differentiable sweep, the
yardstick for the CUDA backward (sphere-stereo_gb300/differentiable.py).  Only tests load it.

Forward, per reference camera (the soft-argmin extension of python/depth_estimation.py:137-198):
  * rays of the reference pixels (python/utils.py:57-73), candidate points d_k * ray;
  * each pixel's selected camera, with its pose perturbed: T_c <- T_c [Exp(omega_c), v_c];
  * projection (python/utils.py:75-94), bilinear zero-padded sample of the camera's image;
  * cost = clamp(sum_ch |sample - reference|, max=500) (depth_estimation.py:173-175);
  * the ISB filter as explicit sparse linear operators for the reference's guide
    (oracle/sphere_oracle.c: sso_isb_operators, float32 weights of the device's arithmetic);
  * q = sum_k softmax(-F_k / temperature) / d_k.
Everything differentiable is float64; torch.autograd gives the gradients with respect to the
images and the 6-DoF pose deltas.  The guide is treated as a constant, as in the device path.
"""
from __future__ import annotations

import numpy as np
import torch

import sphere_oracle as SO


def skew(w: torch.Tensor) -> torch.Tensor:
    z = torch.zeros((), dtype=w.dtype, device=w.device)
    return torch.stack([torch.stack([z, -w[2], w[1]]), torch.stack([w[2], z, -w[0]]),
                        torch.stack([-w[1], w[0], z])])


def so3_exp(w: torch.Tensor) -> torch.Tensor:
    """Rodrigues' formula with series for small angles (differentiable at 0)."""
    th2 = (w * w).sum()
    small = th2 < 1e-12
    th = torch.sqrt(torch.where(small, torch.ones_like(th2), th2))
    a = torch.where(small, 1 - th2 / 6, torch.sin(th) / th)
    b = torch.where(small, 0.5 - th2 / 24, (1 - torch.cos(th)) / torch.where(small, torch.ones_like(th2), th2))
    k = skew(w)
    return torch.eye(3, dtype=w.dtype, device=w.device) + a * k + b * (k @ k)


def perturb(rt: torch.Tensor, delta: torch.Tensor) -> torch.Tensor:
    """T [Exp(omega), v] for delta = (omega, v)."""
    e = torch.eye(4, dtype=rt.dtype, device=rt.device)
    e = torch.cat([torch.cat([so3_exp(delta[:3]), delta[3:, None]], 1), e[3:]], 0)
    return rt @ e


class DiffReference:
    def __init__(self, calibration: dict, *, matching_resolution, min_dist, max_dist, candidate_count,
                 references_indices, selected, guides, sigma_i, sigma_s, temperature, device="cpu"):
        """device: where the float64 evaluation runs (a CUDA device makes the full-size checks
        affordable; the arithmetic is the same float64 on either)."""
        W, H = matching_resolution
        self.W, self.H, self.P = W, H, W * H
        self.refs = list(references_indices)
        self.tau = float(temperature)
        cams32 = SO.parse_calibration(calibration, matching_resolution, torch.float32)
        self.rt = [c["rt"].double() for c in cams32]
        # float32 intrinsics products and candidates, as the device uses them, promoted
        self.k = torch.tensor(np.stack([SO.cam6(c) for c in cams32]), dtype=torch.float64)
        self.cand = (1 / torch.linspace(1 / min_dist, 1 / max_dist, candidate_count)).double()
        self.selected = [torch.as_tensor(np.asarray(s, np.int64)).reshape(-1) for s in selected]
        o = SO.Oracle("f32", exp_mode="device")
        self.ops = []
        for g in guides:
            ops = o.isb_operators(np.asarray(g, np.uint8), sigma_i, sigma_s)
            self.ops.append({k: [torch.as_tensor(np.asarray(a, np.int64 if "idx" in k else np.float64)) for a in v]
                             if k != "shapes" else v for k, v in ops.items()})
        u, v = torch.meshgrid(torch.arange(H, dtype=torch.float64), torch.arange(W, dtype=torch.float64),
                              indexing="ij")
        self.pix = torch.stack([v.reshape(-1), u.reshape(-1)], -1)
        self.device = torch.device(device)
        dev = self.device
        self.rt = [t.to(dev) for t in self.rt]
        self.k, self.cand, self.pix = self.k.to(dev), self.cand.to(dev), self.pix.to(dev)
        self.selected = [t.to(dev) for t in self.selected]
        self.ops = [{k: ([a.to(dev) for a in v] if k != "shapes" else v) for k, v in ops.items()} for ops in self.ops]

    def rays(self, r: int) -> torch.Tensor:
        fx, fy, cx, cy, xi, al = self.k[r]
        mx = (self.pix[:, 0] - cx) / fx
        my = (self.pix[:, 1] - cy) / fy
        r2 = mx * mx + my * my
        mz = (1 - al * al * r2) / (al * torch.sqrt(torch.clamp(1 - (2 * al - 1) * r2, min=0)) + 1 - al)
        s = (mz * xi + torch.sqrt(mz * mz + (1 - xi * xi) * r2)) / (mz * mz + r2)
        return torch.stack([s * mx, s * my, s * mz - xi], -1)

    def sample(self, images: torch.Tensor, sel: torch.Tensor, u: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
        """Bilinear, zero padding; images [C, P, 3]; sel [P]; u, v [N, P] -> [N, P, 3].  Written as
        two horizontal interpolations and a vertical one (the same value as the sum of the four
        weighted taps): four equal taps give exactly their value, so the L1 residual of a sample in
        a flat region is exactly 0 and takes the zero subgradient, as on the device."""
        x0, y0 = torch.floor(u), torch.floor(v)
        fx, fy = (u - x0)[..., None], (v - y0)[..., None]
        taps = []
        for dx, dy in ((0, 0), (1, 0), (0, 1), (1, 1)):
            xs, ys = x0 + dx, y0 + dy
            inb = (xs >= 0) & (xs < self.W) & (ys >= 0) & (ys < self.H)
            idx = (ys.clamp(0, self.H - 1) * self.W + xs.clamp(0, self.W - 1)).long()
            taps.append(images[sel.clamp(min=0)[None].expand_as(idx), idx] * inb[..., None])
        top = taps[0] + fx * (taps[1] - taps[0])
        bot = taps[2] + fx * (taps[3] - taps[2])
        return top + fy * (bot - top)

    def inverse_distance(self, images: torch.Tensor, deltas: torch.Tensor) -> torch.Tensor:
        """images [C, H, W, 3], deltas [C, 6] (float64, on the reference's device) -> q [references, H, W]."""
        C = images.shape[0]
        imgs = images.reshape(C, self.P, 3)
        poses = [perturb(self.rt[c], deltas[c]) for c in range(C)]
        out = []
        for slot, r in enumerate(self.refs):
            rel = torch.stack([torch.linalg.inv(poses[c]) @ poses[r] for c in range(C)])
            sel = self.selected[slot]
            has = sel >= 0
            sc = sel.clamp(min=0)
            ray = self.rays(r)
            p = self.cand[:, None, None] * ray[None]
            R, t = rel[sc, :3, :3], rel[sc, :3, 3]
            q = torch.einsum("pij,npj->npi", R, p) + t[None]
            k = self.k[sc]
            fx, fy, cx, cy, xi, al = (k[:, j][None] for j in range(6))
            x, y, z = q[..., 0], q[..., 1], q[..., 2]
            d1 = torch.sqrt(x * x + y * y + z * z)
            c_ = xi * d1 + z
            d2 = torch.sqrt(x * x + y * y + c_ * c_)
            nrm = al * d2 + (1 - al) * c_
            u = fx * x / nrm + cx
            v = fy * y / nrm + cy
            s = self.sample(imgs, sel, u, v) * has[None, :, None]
            refimg = imgs[r][None]
            cost = torch.clamp(torch.abs(s - refimg).sum(-1), max=500)
            ops = self.ops[slot]
            L = len(ops["shapes"])
            c = [cost]
            for lv in range(1, L):
                c.append((ops["down_w"][lv][None] * c[lv - 1][:, ops["down_idx"][lv]]).sum(-1))
            f = c[L - 1]
            for lv in range(L - 2, -1, -1):
                f = ops["up_own"][lv][None] * c[lv] + (ops["up_w"][lv][None] * f[:, ops["up_idx"][lv]]).sum(-1)
            w = torch.softmax(-f / self.tau, dim=0)
            out.append((w / self.cand[:, None]).sum(0).reshape(self.H, self.W))
        return torch.stack(out)

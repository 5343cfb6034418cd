"""SSIM and the training loss on sm_103a kernels.

A drop-in for the fused-ssim package FasterGS's backbones train with
(gs_submodules/fused-ssim/fused_ssim/__init__.py: ``FusedSSIMMap``,
``fused_ssim``, ``allowed_padding``; called as
``fast_ssim(image.unsqueeze(0), gt_image.unsqueeze(0))`` in
taming-3dgs/train_faster.py:123 and FastGS/train_faster.py:107), and
``l1_dssim_loss``, the whole loss of those training loops
((1 - lambda) l1_loss + lambda (1 - ssim), train_faster.py:121-125) with its
gradient from one fused kernel.  The SSIM is 3DGS's (utils/loss_utils.py:33-63):
11-tap Gaussian window of sigma 1.5, zero padding, C1 = 0.01^2, C2 = 0.03^2.
Tensors are float32 on one CUDA device, last two dimensions (H, W).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._C import _device_of, _f32, _ptr, _stream

allowed_padding = ["same", "valid"]


def _planes(t: torch.Tensor) -> tuple[int, int, int]:
    if t.dim() < 2:
        raise ValueError("SSIM inputs need (..., H, W)")
    H, W = int(t.shape[-2]), int(t.shape[-1])
    return t.numel() // max(H * W, 1), H, W


class FusedSSIMMap(torch.autograd.Function):
    """fused_ssim/__init__.py:8-37: the SSIM map; with train=True the partials the backward needs."""

    @staticmethod
    def forward(ctx, C1, C2, img1, img2, padding="same", train=True):
        dev = _device_of(img1)
        x = _f32("img1", img1, dev)
        y = _f32("img2", img2, dev)
        if x.shape != y.shape:
            raise ValueError("img1 and img2 must have the same shape")
        planes, H, W = _planes(x)
        ssim_map = torch.empty_like(x)
        parts = [torch.empty_like(x) for _ in range(3)] if train else [None, None, None]
        _lib.call("fgs_ssim_fwd", planes, H, W, float(C1), float(C2), _ptr(x), _ptr(y), _ptr(ssim_map),
                  _ptr(parts[0]), _ptr(parts[1]), _ptr(parts[2]), _stream(dev))
        if padding == "valid":
            ssim_map = ssim_map[..., 5:-5, 5:-5]
        ctx.save_for_backward(x.detach(), y, *(p if p is not None else torch.empty(0) for p in parts))
        ctx.padding = padding
        ctx.train = train
        return ssim_map

    @staticmethod
    def backward(ctx, opt_grad):
        if not ctx.train:
            raise RuntimeError("fused_ssim was called with train=False: no partials were kept")
        x, y, d_mu1, d_e11, d_e12 = ctx.saved_tensors
        dev = x.device
        g = opt_grad
        if ctx.padding == "valid":
            g = torch.zeros_like(x)
            g[..., 5:-5, 5:-5] = opt_grad
        g = _f32("dL_dmap", g, dev)
        planes, H, W = _planes(x)
        grad = torch.empty_like(x)
        _lib.call("fgs_ssim_bwd", planes, H, W, _ptr(x), _ptr(y), _ptr(g), _ptr(d_mu1), _ptr(d_e11), _ptr(d_e12),
                  _ptr(grad), _stream(dev))
        return None, None, grad, None, None, None


def fused_ssim(img1, img2, padding="same", train=True):
    """fused_ssim/__init__.py:39-46: mean SSIM of img1 against img2 (differentiable in img1)."""
    C1 = 0.01 ** 2
    C2 = 0.03 ** 2
    assert padding in allowed_padding
    ssim_map = FusedSSIMMap.apply(C1, C2, img1, img2, padding, train)
    return ssim_map.mean()


_SCRATCH: dict = {}


def _scratch(dev, nbytes: int) -> torch.Tensor:
    key = (dev.type, dev.index)
    buf = _SCRATCH.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(nbytes, 8), dtype=torch.uint8, device=dev)
        _SCRATCH[key] = buf
    return buf


class _L1DSSIM(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, gt, lambda_dssim):
        dev = _device_of(image)
        x = _f32("image", image, dev)
        y = _f32("gt", gt, dev)
        if x.shape != y.shape:
            raise ValueError("image and gt must have the same shape")
        planes, H, W = _planes(x)
        nbytes = int(_lib.load().fgs_l1_dssim_scratch_bytes(planes, H, W))
        if nbytes == 0:
            raise ValueError("image too large or empty")
        scratch = _scratch(dev, nbytes)
        out = torch.empty(2, dtype=torch.float32, device=dev)  # loss, mean SSIM
        grad = torch.empty_like(x)
        _lib.call("fgs_l1_dssim", planes, H, W, float(lambda_dssim), _ptr(x), _ptr(y), scratch.data_ptr(),
                  scratch.numel(), out.data_ptr(), out.data_ptr() + 4, _ptr(grad), _stream(dev))
        ctx.save_for_backward(grad)
        loss, ssim_mean = out[0].clone(), out[1].clone()
        ctx.mark_non_differentiable(ssim_mean)
        return loss, ssim_mean

    @staticmethod
    def backward(ctx, grad_loss, _grad_ssim):
        grad, = ctx.saved_tensors
        return grad * grad_loss, None, None


def l1_dssim_loss(image, gt, lambda_dssim: float = 0.2):
    """(1 - lambda) mean|image - gt| + lambda (1 - mean SSIM(image, gt)) and the mean SSIM, the
    loss of train_faster.py:121-125 in one fused pass; the gradient w.r.t. image is produced by the
    same kernel and handed to autograd.  Returns (loss, ssim_mean), 0-dim tensors."""
    return _L1DSSIM.apply(image, gt, lambda_dssim)

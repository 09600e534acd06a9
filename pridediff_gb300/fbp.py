"""FBP filtering on the GPU.

deeprecon's filtered_backprojection (deeprecon/torch/projector/projector.py:
192-213 for 2-D, 368-390 for cone beams, 554-563 for spirals) weights the
sinogram by the cosine weight and filters every detector row with a
2 num_det - 1 tap kernel through ``nn.functional.conv2d`` / ``conv3d`` with
padding num_det - 1, before the weighted DD back-projection.  Here both steps
are one CUDA kernel (``dd_fbp_filter``: the weight is applied as the rows are
staged, the cross-correlation runs in FP32 on the staged rows).

``FbpFilter`` carries the gradient with respect to the sinogram (the same
kernel with the taps reversed, then the weight).  A trainable weight or
filter (``trainable=True``) keeps the torch convolution so that autograd
reaches them.
"""
from __future__ import annotations

import torch
from torch import Tensor

from . import _native as N


def _launch(x: Tensor, out: Tensor, weight, wrows: int, taps: Tensor) -> None:
    lib = N.load()
    D = x.shape[-1]
    rows = x.numel() // D
    stream = torch.cuda.current_stream(x.device).cuda_stream
    st = lib.dd_fbp_filter(x.data_ptr(), out.data_ptr(), weight.data_ptr() if weight is not None else None,
                           wrows, taps.data_ptr(), rows, D, stream)
    N.check(st, "dd_fbp_filter")


class FbpFilter(torch.autograd.Function):
    """out = correlate(sino * weight, taps) along the last dimension."""

    @staticmethod
    def forward(ctx, sino: Tensor, weight: Tensor, taps: Tensor) -> Tensor:
        sino = sino.contiguous()
        out = torch.empty_like(sino)
        _launch(sino, out, weight, weight.numel() // sino.shape[-1], taps)
        ctx.save_for_backward(weight, taps)
        return out

    @staticmethod
    def backward(ctx, grad: Tensor):
        weight, taps = ctx.saved_tensors
        grad = grad.contiguous()
        g = torch.empty_like(grad)
        _launch(grad, g, None, 1, taps.flip(0).contiguous())
        return g * weight, None, None


def fused_ok(sino: Tensor, weight: Tensor, taps: Tensor) -> bool:
    """The fused kernel applies: CUDA data, a 2D - 1 tap filter, and neither
    the weight nor the filter asks for a gradient."""
    D = sino.shape[-1]
    return (sino.is_cuda and taps.numel() == 2 * D - 1 and weight.shape[-1] == D
            and not (weight.requires_grad or taps.requires_grad))


def weighted_filter(sino: Tensor, weight: Tensor, taps: Tensor) -> Tensor:
    """``conv(sino * weight, taps, padding=D - 1)`` over the detector bins."""
    dev = sino.device
    w = weight.detach().to(dev, torch.float32).contiguous()
    t = taps.detach().reshape(-1).to(dev, torch.float32).contiguous()
    return FbpFilter.apply(sino.to(torch.float32), w, t)

"""PrideDiff's data-consistency block on this library (model/pridediff.py:9-68).

PrideDiff builds one fan-arc projector (512^2 pixels of 0.7433 mm, 768
detectors of 1.2858 mm, iso_source 595, source_detector 490.6, 720 views
over 2 pi), takes A = projection and AT = filtered_backprojection, wraps them
in autograd Functions whose backward is the other operator (``prj_fun``:
forward A, backward FBP; ``prj_t_fun``: forward FBP, backward A) and computes

    out = x - w * AT(A x - y)

with one learned scalar w (``fidelity_module``).  ``FidelityModule`` keeps
that behaviour (``adjoint="fbp"``) or uses the exact matched adjoint instead
(``adjoint="exact"``: AT = ProjTrans, so that w * AT(A x - y) is a gradient
step on ||A x - y||^2 / 2 and the backward of A is its true transpose).
``fidelity_graph`` captures steps of the block in one CUDA graph, as a
sampling loop would replay it between network evaluations.
"""
from __future__ import annotations

import torch
import torch.nn as nn
from torch.autograd import Function

from .projector import projector2d


def pridediff_projector() -> projector2d:
    """The projector model/pridediff.py:9-14 builds."""
    return projector2d(image_size=512, num_det=768, pix_size=0.7433, det_size=1.2858, iso_source=595.0,
                       source_detector=490.6, scan_type="arc")


def pridediff_views(device=None) -> torch.Tensor:
    """model/pridediff.py:16: 720 views over 2 pi."""
    return torch.arange(720, device=device) * torch.pi * 2 / 720


class _Prj(Function):
    """prj_fun: forward A, backward the module's adjoint (FBP in PrideDiff)."""

    @staticmethod
    def forward(ctx, image, mod):
        ctx.mod = mod
        return mod.proj.projection(image, mod.views)

    @staticmethod
    def backward(ctx, grad):
        return ctx.mod.adjoint_op(grad.contiguous()), None


class _PrjT(Function):
    """prj_t_fun: forward the module's adjoint, backward A."""

    @staticmethod
    def forward(ctx, sino, mod):
        ctx.mod = mod
        return mod.adjoint_op(sino)

    @staticmethod
    def backward(ctx, grad):
        return ctx.mod.proj.projection(grad.contiguous(), ctx.mod.views), None


class FidelityModule(nn.Module):
    """out = x - weight * AT(A x - proj).

    proj / views default to PrideDiff's projector and views; adjoint is
    "fbp" (PrideDiff: filtered_backprojection) or "exact" (ProjTrans).
    PrideDiff allocates the weight uninitialised and loads it from a
    checkpoint; here it starts at 0 until set or loaded (its state_dict key
    is ``weight``, as in PrideDiff; the projector's tensors sit under
    ``proj.``).
    """

    def __init__(self, proj: projector2d = None, views: torch.Tensor = None, adjoint: str = "fbp"):
        super().__init__()
        if adjoint not in ("fbp", "exact"):
            raise ValueError(f"adjoint must be 'fbp' or 'exact', not {adjoint!r}")
        self.weight = nn.Parameter(torch.zeros(()))
        self.proj = proj if proj is not None else pridediff_projector()
        self.register_buffer("views", views if views is not None else pridediff_views(), persistent=False)
        self.adjoint = adjoint

    def adjoint_op(self, sino: torch.Tensor) -> torch.Tensor:
        if self.adjoint == "fbp":
            return self.proj.filtered_backprojection(sino, self.views)
        return self.proj.projection_t(sino, self.views)

    def forward(self, input_data: torch.Tensor, proj: torch.Tensor, t=None) -> torch.Tensor:
        temp = _Prj.apply(input_data, self) - proj
        intervening_res = _PrjT.apply(temp, self)
        return input_data - self.weight * intervening_res


def fidelity_graph(module: FidelityModule, x: torch.Tensor, y: torch.Tensor, steps: int = 1):
    """Capture `steps` applications x <- module(x, y) (in place, no autograd)
    in one CUDA graph; replay it to run them."""
    with torch.no_grad():
        module(x.clone(), y)   # warm-up: plans, tables and kernel attributes
    torch.cuda.synchronize(x.device)
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream(x.device)
    s.wait_stream(torch.cuda.current_stream(x.device))
    with torch.no_grad(), torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            for _ in range(steps):
                x.copy_(module(x, y))
    torch.cuda.current_stream(x.device).wait_stream(s)
    return graph


class GraphedFidelity:
    """One application of a FidelityModule, x -> x - w * AT(A x - y), replayed
    from a CUDA graph captured once: the data-consistency step of a sampling
    loop, called between evaluations of a network that stays in stock
    PyTorch (GaussianDiffusion.sample calls it through learn_block at every
    step, model/pridediff.py:276-277).

    The graph reads a static input and a static sinogram and writes a static
    output; ``set_sino`` loads the measured sinogram once per sampling run and
    each call copies x in, replays and returns a copy of the output.  The
    module's weight is read by the graph where it lies, so loading another
    weight in place needs no recapture."""

    def __init__(self, module: FidelityModule, x_like: torch.Tensor, sino_like: torch.Tensor):
        self.module = module
        self.x = torch.zeros_like(x_like)
        self.y = torch.zeros_like(sino_like)
        with torch.no_grad():
            module(self.x, self.y)   # warm-up: plans, tables and kernel attributes
        torch.cuda.synchronize(self.x.device)
        self.graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.x.device)
        s.wait_stream(torch.cuda.current_stream(self.x.device))
        with torch.no_grad(), torch.cuda.stream(s):
            with torch.cuda.graph(self.graph, stream=s):
                self.out = module(self.x, self.y)
        torch.cuda.current_stream(self.x.device).wait_stream(s)

    def set_sino(self, sino: torch.Tensor) -> None:
        self.y.copy_(sino)

    def __call__(self, x: torch.Tensor, sino=None, t=None) -> torch.Tensor:
        self.x.copy_(x)
        self.graph.replay()
        return self.out.clone()


def sample(denoise_fn, learn_block, img: torch.Tensor, sino: torch.Tensor, alphas: torch.Tensor,
           steps: int = None):
    """GaussianDiffusion.sample (model/pridediff.py:256-298): from t = steps
    down to 1, x1 = learn_block(denoise_fn(img, t - 1), sino, max(t - 2, 0)),
    then img <- img - q(x1, t - 1) + q(x1, t - 2) with q(x, s) = a_s x +
    (1 - a_s) noise (q_sample, :300-305; the last step uses x1 itself).
    `learn_block(x, sino, t)` carries the data-consistency step (a
    GraphedFidelity inside it replays it from a CUDA graph).  Returns (the
    input, the first step's reconstruction, the final image), as the
    reference does."""
    b = img.shape[0]
    t = int(alphas.numel()) if steps is None else int(steps)
    noise, xt, direct = img, img, None

    def q(x, s):
        a = alphas.gather(-1, s).reshape(b, *((1,) * (x.dim() - 1)))
        return a * x + (1.0 - a) * noise

    with torch.no_grad():
        while t:
            step = torch.full((b,), t - 1, dtype=torch.long, device=img.device)
            step2 = torch.full((b,), max(t - 2, 0), dtype=torch.long, device=img.device)
            x1 = learn_block(denoise_fn(img, step), sino, step2)
            if direct is None:
                direct = x1
            xt_bar = q(x1, step)
            xt_sub1 = q(x1, step2) if t - 1 != 0 else x1
            img = img - xt_bar + xt_sub1
            t -= 1
    return xt, direct, img


__all__ = ["FidelityModule", "GraphedFidelity", "fidelity_graph", "pridediff_projector", "pridediff_views",
           "sample"]

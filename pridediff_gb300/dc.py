"""Data-consistency (DC) pieces for diffusion sampling and unrolled networks.

PrideDiff's DC module computes x - w * AT(A x - y) from two separate operator
calls and lets autograd keep the residual (model/pridediff.py:56-68, with FBP
standing in for the adjoint).  Here:

* ``dc_loss(proj, x, y, angles)``: ||A x - y||^2 as an autograd Function whose
  backward is the exact matched adjoint, 2 A^T (A x - y) * grad.  The
  sinogram-sized residual is not saved between forward and backward; the
  backward recomputes it with one fused forward (A x - y written directly).
* ``dc_step(proj, x, y, angles, eta)``: x <- x - eta * A^T (A x - y) in place,
  fused (dd2d_dc_step), and ``dc_step_graph`` capturing many of them in one
  CUDA graph.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N
from . import status as _status
from .radontorch import _stream_ptr, host_options, plan2d


def _geom(proj):
    return N.geom2d(host_options(proj.options))


def residual(proj, x: torch.Tensor, y: torch.Tensor, angles: torch.Tensor) -> torch.Tensor:
    """A x - y in one fused launch (no separate subtraction pass)."""
    lib = N.load()
    g = _geom(proj)
    x = x.contiguous()
    y = y.contiguous()
    B = x.shape[0] * x.shape[1]
    V = int(angles.shape[0])
    N.check(lib.dd2d_validate(N.SCAN2D[proj.scan_type], N.OPS["proj"], g, B, V), "residual")
    plan = plan2d(proj.scan_type, g, angles)
    out = torch.empty_like(y)
    nbytes = int(lib.dd2d_dc_workspace_bytes(N.SCAN2D[proj.scan_type], g, B, V))
    ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
    # dd2d_dc_step with eta = 0 leaves x unchanged and writes A x - y into `out`
    _status.check(x.device)
    with torch.cuda.device(x.device):
        st = lib.dd2d_dc_step(N.SCAN2D[proj.scan_type], g, plan.data_ptr(), x.data_ptr(), y.data_ptr(),
                              out.data_ptr(), 0.0, B, V, ws.data_ptr(), nbytes, _stream_ptr(x.device))
    N.check(st, "residual")
    return out


class _DCLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, proj, angles):
        r = residual(proj, x, y, angles)
        ctx.save_for_backward(x, y)   # inputs only: the residual is recomputed
        ctx.proj, ctx.angles = proj, angles
        return (r.double() ** 2).sum().float()

    @staticmethod
    def backward(ctx, grad):
        x, y = ctx.saved_tensors
        r = residual(ctx.proj, x, y, ctx.angles)
        gx = ctx.proj.projection_t(r, ctx.angles) * (2.0 * grad)
        return gx, None, None, None


def dc_loss(proj, x: torch.Tensor, y: torch.Tensor, angles: torch.Tensor) -> torch.Tensor:
    """||A x - y||^2 with the exact adjoint in backward and no stored residual."""
    return _DCLoss.apply(x, y, proj, angles)


def dc_step(proj, x: torch.Tensor, y: torch.Tensor, angles: torch.Tensor, eta: float,
            resid: torch.Tensor = None, workspace: torch.Tensor = None) -> torch.Tensor:
    """In place: x <- x - eta * A^T (A x - y) (fused forward + exact adjoint)."""
    lib = N.load()
    g = _geom(proj)
    B = x.shape[0] * x.shape[1]
    V = int(angles.shape[0])
    sc = N.SCAN2D[proj.scan_type]
    N.check(lib.dd2d_validate(sc, N.OPS["proj"], g, B, V), "dc step")
    if not (x.is_contiguous() and y.is_contiguous()):
        raise RuntimeError("dc_step needs contiguous x and y")
    plan = plan2d(proj.scan_type, g, angles)
    if resid is None:
        resid = torch.empty_like(y)
    nbytes = int(lib.dd2d_dc_workspace_bytes(sc, g, B, V))
    if workspace is None or workspace.numel() < nbytes:
        workspace = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
    _status.check(x.device)
    with torch.cuda.device(x.device):
        st = lib.dd2d_dc_step(sc, g, plan.data_ptr(), x.data_ptr(), y.data_ptr(), resid.data_ptr(), float(eta),
                              B, V, workspace.data_ptr(), workspace.numel(), _stream_ptr(x.device))
    N.check(st, "dc step")
    return x


def dc_step_graph(proj, x: torch.Tensor, y: torch.Tensor, angles: torch.Tensor, eta: float, steps: int):
    """Capture `steps` fused DC steps on (x, y) in one CUDA graph (x updated in place)."""
    resid = torch.empty_like(y)
    lib = N.load()
    g = _geom(proj)
    nbytes = int(lib.dd2d_dc_workspace_bytes(N.SCAN2D[proj.scan_type], g, x.shape[0] * x.shape[1],
                                             int(angles.shape[0])))
    ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
    dc_step(proj, x.clone(), y, angles, 0.0, resid, ws)   # warm-up: plan and kernel attributes
    torch.cuda.synchronize(x.device)
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream(x.device)
    s.wait_stream(torch.cuda.current_stream(x.device))
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            for _ in range(steps):
                dc_step(proj, x, y, angles, eta, resid, ws)
    torch.cuda.current_stream(x.device).wait_stream(s)
    graph._pridediff_keep = (resid, ws)   # buffers the graph uses
    return graph

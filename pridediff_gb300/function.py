"""Autograd pairs of the DD operators (drop-in for deeprecon's function.py).

Each Function pairs an operator with its exact transpose, as
deeprecon/deeprecon/torch/projector/function.py:7-532 does:

* ``Proj*``           backward -> ``ProjTrans*``      (A  <-> A^T)
* ``ProjTrans*``      backward -> ``Proj*``
* ``BackProj*``       backward -> ``BackProjTrans*``  (B  <-> B^T)
* ``BackProjTrans*``  backward -> ``BackProj*``
* ``BackProjWeighted*`` backward -> ``BackProjTransWeighted*``

Inputs are cast to float32 under autocast (``custom_fwd(cast_inputs=float32)``
in the reference); only ``(options, angles[, source_pos])`` are saved -- the
backward never needs the forward input or output, so nothing of the size of
an image or sinogram is kept alive between forward and backward.  The
gradients for options, angles and source_pos are ``None``.
"""
from __future__ import annotations

import torch
from torch.autograd import Function

from . import radontorch

try:  # torch >= 2.4
    from torch.amp import custom_bwd as _cbwd, custom_fwd as _cfwd

    def _fwd(fn):
        return _cfwd(device_type="cuda", cast_inputs=torch.float32)(fn)

    def _bwd(fn):
        return _cbwd(device_type="cuda")(fn)
except ImportError:  # pragma: no cover
    from torch.cuda.amp import custom_bwd as _bwd0, custom_fwd as _cfwd0

    def _fwd(fn):
        return _cfwd0(cast_inputs=torch.float32)(fn)

    def _bwd(fn):
        return _bwd0(fn)


def _make(name: str, fwd_op: str, bwd_op: str, spiral: bool):
    fop = getattr(radontorch, fwd_op)
    bop = getattr(radontorch, bwd_op)

    if spiral:
        class _F(Function):
            @staticmethod
            @_fwd
            def forward(ctx, input, option, angles, source_pos):
                output = fop(input.contiguous(), option, angles, source_pos)
                ctx.save_for_backward(option, angles, source_pos)
                return output

            @staticmethod
            @_bwd
            def backward(ctx, grad_output):
                return bop(grad_output.contiguous(), *ctx.saved_tensors), None, None, None
    else:
        class _F(Function):
            @staticmethod
            @_fwd
            def forward(ctx, input, option, angles):
                output = fop(input.contiguous(), option, angles)
                ctx.save_for_backward(option, angles)
                return output

            @staticmethod
            @_bwd
            def backward(ctx, grad_output):
                return bop(grad_output.contiguous(), *ctx.saved_tensors), None, None

    _F.__name__ = _F.__qualname__ = name
    _F.__doc__ = f"{fwd_op} with backward {bwd_op} (deeprecon function.py)."
    return _F


_PAIRS = [("Proj", "ProjTrans"), ("ProjTrans", "Proj"), ("BackProj", "BackProjTrans"),
          ("BackProjTrans", "BackProj"), ("BackProjWeighted", "BackProjTransWeighted")]

__all__ = []
for _geo, _suffix, _weighted in (("FanFlat", "Dis2d", True), ("FanArc", "Dis2d", True),
                                 ("Para", "Dis2d", False), ("ConeFlat", "Dis3d", True),
                                 ("ConeArc", "Dis3d", True), ("Spiral", "Dis3d", True)):
    for _a, _b in _PAIRS:
        if _a == "BackProjWeighted" and not _weighted:
            continue
        _name = f"{_a}{_geo}{_suffix}"
        globals()[_name] = _make(_name, _name, f"{_b}{_geo}{_suffix}", _geo == "Spiral")
        __all__.append(_name)


def _sysmatrix(op_name):
    def f(option, angles):
        # the reference forces CPU float32 here (function.py:535-553)
        return getattr(radontorch, op_name)(option, angles)
    f.__name__ = op_name
    return f


GetSysMatrixFanFlat2d = _sysmatrix("GetSysMatrixFanFlat2d")
GetSysMatrixFanArc2d = _sysmatrix("GetSysMatrixFanArc2d")
GetSysMatrixPara2d = _sysmatrix("GetSysMatrixPara2d")
__all__ += ["GetSysMatrixFanFlat2d", "GetSysMatrixFanArc2d", "GetSysMatrixPara2d"]

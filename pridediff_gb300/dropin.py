"""Make code written against deeprecon run on this package, unchanged.

deeprecon's projector modules import its compiled extension under the name
``radontorch`` (``deeprecon/torch/projector/function.py:2``), and PrideDiff
imports the projector classes as ``from deeprecon.torch.projector import
projector2d`` (``model/pridediff.py:7``, ``model/diffusion.py:7``).

``install()`` registers this package's ``radontorch`` under that name, so an
installed deeprecon runs its own Python layer on these kernels.  Where
deeprecon itself is not installed (or ``projector=True``), it also registers
the module path ``deeprecon.torch.projector`` -- with ``projector``,
``function`` and ``filter`` submodules -- served by this package's modules,
so PrideDiff's imports resolve to ``pridediff_gb300.projector``.  Call it
before the first import of deeprecon.  Returns the names it registered.
"""
from __future__ import annotations

import importlib.util
import sys
import types
from typing import List


def _module(name: str, package: bool = True) -> types.ModuleType:
    m = types.ModuleType(name)
    if package:
        m.__path__ = []   # a namespace for the submodules registered below
    return m


def install(projector: bool = False) -> List[str]:
    from . import filter as _filter
    from . import function as _function
    from . import projector as _projector
    from . import radontorch as _radontorch

    sys.modules["radontorch"] = _radontorch
    names = ["radontorch"]
    if not projector and importlib.util.find_spec("deeprecon") is not None:
        return names
    root = _module("deeprecon")
    torch_pkg = _module("deeprecon.torch")
    proj_pkg = _module("deeprecon.torch.projector")
    for cls in ("projector2d", "projector3d", "projectorsp"):
        setattr(proj_pkg, cls, getattr(_projector, cls))
    proj_pkg.projector = _projector
    proj_pkg.function = _function
    proj_pkg.filter = _filter
    torch_pkg.projector = proj_pkg
    root.torch = torch_pkg
    mods = {"deeprecon": root, "deeprecon.torch": torch_pkg, "deeprecon.torch.projector": proj_pkg,
            "deeprecon.torch.projector.projector": _projector,
            "deeprecon.torch.projector.function": _function,
            "deeprecon.torch.projector.filter": _filter}
    sys.modules.update(mods)
    return names + list(mods)

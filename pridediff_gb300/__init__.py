"""GB300-native distance-driven CT projector.

Drop-in for the DD forward/back-projection operators of deeprecon (the CT
library inside phoenixyu/PrideDiff): the same projector modules, autograd
pairs and ``radontorch`` operator names, computed by hand-written sm_103a
CUDA kernels in ``libpridediff_dd.so`` through a plain C ABI
(``include/pridediff_dd.h``).
"""
from . import _native
from . import radontorch
from .projector import projector2d, projector3d, projectorsp
from .status import device_status

__all__ = ["projector2d", "projector3d", "projectorsp", "radontorch", "build", "device_status"]


def build(force: bool = False) -> str:
    """Compile the CUDA library for sm_103a (idempotent)."""
    return _native.build(force=force)

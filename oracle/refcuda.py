"""deeprecon's own CUDA kernels, called the way radontorch calls them --
TEST INFRASTRUCTURE.

The kernels are the reference's device code, compiled unmodified from
``deeprecon/cuda/dis{2,3}d/*.cu`` into ``_ref/cuda/*.fatbin`` by ``make``
where the reference sources exist; ``_build/libddrefcuda.so``
(``ref_cuda_host.cpp``) launches them with the reference host functions'
texture staging, grids and default stream.  Only ``tests/`` (the 3-D parity
checker), ``tests/golden/make_golden.py`` (fixtures) and ``bench.py`` (the
plain-GPU comparator) use this module.

``run(geom, op, x, angles, options, source_pos)`` mirrors one radontorch call
(``interface/RadonTorch.cpp``): x is a CUDA tensor (B, C, ...), the output is
allocated like the reference allocates it (``torch::zeros`` for the
accumulating operators, ``torch::empty`` otherwise) and returned.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
FATBIN_DIR = os.path.join(_HERE, "_ref", "cuda")
_LIB = os.path.join(_HERE, "_build", "libddrefcuda.so")
_FILES = ("ParaDisCUDA2d", "FanFlatDisCUDA2d", "FanArcDisCUDA2d", "ConeFlatDisCUDA3d",
          "ConeArcDisCUDA3d", "SpiralDisCUDA3d")

GEOM = {"para": 0, "flat": 1, "arc": 2, "cone_flat": 3, "cone_arc": 4, "spiral": 5}
OPS = {"proj": 0, "proj_t": 1, "bproj": 2, "bproj_t": 3, "bproj_w": 4, "bproj_tw": 5}
IMAGE_INPUT = {"proj", "bproj_t", "bproj_tw"}
# operators whose radontorch host function allocates the output with torch::zeros
# and accumulates into it (RadonTorch.cpp:68, :98, :158 and their 3-D twins)
ZEROED = {"proj_t", "bproj", "bproj_w"}

_lib = None


def available() -> bool:
    """True where the reference fatbins were built (they need the reference sources)."""
    return all(os.path.exists(os.path.join(FATBIN_DIR, f + ".fatbin")) for f in _FILES)


def _load():
    global _lib
    if _lib is None:
        if not available():
            raise FileNotFoundError("reference CUDA fatbins absent (oracle/_ref/cuda)")
        if not os.path.exists(_LIB):
            import oracle
            oracle.build()
        lib = ctypes.CDLL(_LIB)
        lib.refcuda_last_error.restype = ctypes.c_char_p
        lib.refcuda_load.restype = ctypes.c_int
        lib.refcuda_load.argtypes = [ctypes.c_char_p]
        lib.refcuda_run.restype = ctypes.c_int
        lib.refcuda_run.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 + \
            [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)]
        _lib = lib
    import torch
    torch.cuda.init()
    if _lib.refcuda_load(FATBIN_DIR.encode()) != 0:
        raise RuntimeError("refcuda_load: " + _lib.refcuda_last_error().decode())
    return _lib


def _split_options(geom: str, options):
    o = np.asarray(options.detach().cpu() if hasattr(options, "detach") else options,
                   dtype=np.float32).reshape(-1)
    if geom in ("para", "flat", "arc"):
        if o.size != 11:
            raise ValueError("2-D options must have 11 entries")
        return [int(v) for v in o[:3]], [float(v) for v in o[3:11]]
    n = 16 if geom == "spiral" else 17
    if o.size != n:
        raise ValueError(f"{geom} options must have {n} entries")
    return [int(v) for v in o[:5]], [float(v) for v in o[5:n]]


def out_shape(geom: str, op: str, shape, options, nview: int):
    ints, _ = _split_options(geom, options)
    b, c = int(shape[0]), int(shape[1])
    if geom in ("para", "flat", "arc"):
        w, h, nd = ints
        return (b, c, nview, nd) if op in IMAGE_INPUT else (b, c, h, w)
    w, h, d, ncol, nrow = ints
    return (b, c, nview, nrow, ncol) if op in IMAGE_INPUT else (b, c, d, h, w)


def run(geom: str, op: str, x, angles, options, source_pos=None):
    """One reference operator call on CUDA tensors; returns a new CUDA tensor."""
    import torch
    lib = _load()
    if not (x.is_cuda and angles.is_cuda):
        raise ValueError("refcuda.run takes CUDA tensors")
    x = x.contiguous().float()
    angles = angles.contiguous().float()
    nview = int(angles.numel())
    ints, floats = _split_options(geom, options)
    shape = out_shape(geom, op, x.shape, options, nview)
    out = (torch.zeros if op in ZEROED else torch.empty)(shape, device=x.device, dtype=torch.float32)
    batch = int(x.shape[0]) * int(x.shape[1])
    if geom in ("para", "flat", "arc"):
        w, h, nd = ints
        iv = [w, h, nview, nd]
    else:
        w, h, d, ncol, nrow = ints
        iv = [w, h, d, nview, ncol, nrow]
    sp_ptr = None
    if geom == "spiral":
        if source_pos is None or tuple(source_pos.shape) != (4, nview) or not source_pos.is_cuda:
            raise ValueError("spiral needs a (4, V) CUDA source_pos")
        source_pos = source_pos.contiguous().float()
        sp_ptr = source_pos.data_ptr()
    ia = (ctypes.c_int * 6)(*iv)
    fa = (ctypes.c_float * 12)(*floats)
    # the reference launches on the legacy default stream; order it after torch's work
    if torch.cuda.current_stream() != torch.cuda.default_stream():
        torch.cuda.current_stream().synchronize()
    rc = lib.refcuda_run(GEOM[geom], OPS[op], out.data_ptr(), x.data_ptr(), angles.data_ptr(), sp_ptr,
                         batch, ia, fa)
    if rc != 0:
        raise RuntimeError(f"reference CUDA {geom}/{op}: " + lib.refcuda_last_error().decode())
    return out

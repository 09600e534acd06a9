"""CPU oracle for the distance-driven projector -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package.  It is the checker, never the product: the
product path (``pridediff_gb300``) has no CPU fallback and never imports it.

Two back ends:

* ``run2d`` / ``run3d`` call ``_build/libddoracle.so``, a C restatement of
  deeprecon's distance-driven walk (``ddoracle_body.h``) at FP32 (``prec='f'``,
  the parity oracle that reproduces the reference's FP32 rounding, also the
  timed CPU "port") or FP64 (``prec='d'``).
* ``ref2d`` / ``ref_sysmatrix`` call ``_ref/libddref.so``, deeprecon's own CPU
  projectors compiled unmodified from the reference sources (2-D only; the
  reference has no CPU path for 3-D).  It exists only where the reference
  sources were present at build time; ``have_ref()`` says whether it does.

Geometry is passed as deeprecon's ``options`` vector (11 entries for 2-D,
``projector.py:113``; 17 for cone, ``projector.py:286``; 16 for spiral,
``projector.py:460``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libddoracle.so")
_REF = os.path.join(_HERE, "_ref", "libddref.so")

GEOM2 = {"para": 0, "flat": 1, "arc": 2}
GEOM3 = {"cone_flat": 0, "cone_arc": 1, "spiral": 2}
OPS = {
    "proj": 0,       # Proj*           image -> sinogram (A)
    "proj_t": 1,     # ProjTrans*      sinogram -> image (A^T)
    "bproj": 2,      # BackProj*       sinogram -> image (DD-BP)
    "bproj_t": 3,    # BackProjTrans*  image -> sinogram
    "bproj_w": 4,    # BackProjWeighted*
    "bproj_tw": 5,   # BackProjTransWeighted*
}
IMAGE_INPUT = {"proj", "bproj_t", "bproj_tw"}


class _Geom2(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("nd", ctypes.c_int),
                ("nv", ctypes.c_int)] + [(n, ctypes.c_double) for n in (
                    "pix_x", "pix_y", "det_size", "iso_source", "source_detector",
                    "pix_xshift", "pix_yshift", "bin_shift")]


class _Geom3(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("width", "height", "depth", "ncol", "nrow", "nv")] + \
               [(n, ctypes.c_double) for n in (
                   "pix_x", "pix_y", "pix_z", "col_size", "row_size", "iso_source",
                   "source_detector", "pix_xshift", "pix_yshift", "pix_zshift", "col_shift",
                   "row_shift")]


_lib = None
_ref = None


def build(quiet: bool = True) -> None:
    """Compile the oracle (and the reference, where its sources exist)."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        lib = ctypes.CDLL(_LIB)
        for pre, ct in (("f", ctypes.c_float), ("d", ctypes.c_double)):
            f2 = getattr(lib, f"ddo_{pre}_ddo_run2d")
            f2.restype = ctypes.c_int
            f2.argtypes = [ctypes.POINTER(_Geom2), ctypes.c_int, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ct),
                           ctypes.POINTER(ct), ctypes.c_int, ctypes.c_int]
            f3 = getattr(lib, f"ddo_{pre}_ddo_run3d")
            f3.restype = ctypes.c_int
            f3.argtypes = [ctypes.POINTER(_Geom3), ctypes.c_int, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                           ctypes.POINTER(ct), ctypes.POINTER(ct), ctypes.c_int, ctypes.c_int]
        lib.ddo_f_ddo_scan2d.restype = ctypes.c_longlong
        lib.ddo_f_ddo_scan2d.argtypes = [ctypes.POINTER(_Geom2), ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_float), ctypes.c_double,
                                         ctypes.POINTER(ctypes.c_int)]
        lib.ddo_f_ddo_scan3d.restype = ctypes.c_longlong
        lib.ddo_f_ddo_scan3d.argtypes = [ctypes.POINTER(_Geom3), ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_float),
                                         ctypes.POINTER(ctypes.c_float), ctypes.c_double,
                                         ctypes.POINTER(ctypes.c_int)]
        lib.ddo_default_threads.restype = ctypes.c_int
        lib.ddo_default_threads.argtypes = [ctypes.c_int]
        _lib = lib
    return _lib


def have_ref() -> bool:
    return os.path.exists(_REF)


def _load_ref():
    global _ref
    if _ref is None:
        if not have_ref():
            raise FileNotFoundError("reference CPU build absent (oracle/_ref/libddref.so)")
        _ref = ctypes.CDLL(_REF)
        _ref.ref_sysmatrix.restype = ctypes.c_int64
        _ref.ref_sysmatrix.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_float)] + \
            [ctypes.c_int] * 4 + [ctypes.c_float] * 8 + \
            [ctypes.POINTER(ctypes.POINTER(ctypes.c_int64))] * 2 + \
            [ctypes.POINTER(ctypes.POINTER(ctypes.c_float))]
        _ref.ref_free.argtypes = [ctypes.c_void_p]
    return _ref


def default_threads(nv: int) -> int:
    return int(_load().ddo_default_threads(int(nv)))


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def geom2_from_options(options, nv: int) -> _Geom2:
    o = [float(x) for x in np.asarray(options, dtype=np.float32).reshape(-1)]
    if len(o) != 11:
        raise ValueError("2-D options must have 11 entries")
    return _Geom2(int(o[0]), int(o[1]), int(o[2]), int(nv), *o[3:11])


def geom3_from_options(options, nv: int, spiral: bool = False) -> _Geom3:
    o = [float(x) for x in np.asarray(options, dtype=np.float32).reshape(-1)]
    if spiral:
        if len(o) != 16:
            raise ValueError("spiral options must have 16 entries")
        # (W,H,D, C,R, sx,sy,sz, dc,dr, R,SDD, px,py, cs,rs): no z shift
        o = o[:14] + [0.0] + o[14:]
    elif len(o) != 17:
        raise ValueError("3-D options must have 17 entries")
    return _Geom3(*(int(x) for x in o[:5]), int(nv), *o[5:17])


def _out_shape2(g: _Geom2, op: str, batch: int):
    return (batch, g.nv, g.nd) if op in IMAGE_INPUT else (batch, g.height, g.width)


def run2d(geom: str, op: str, x: np.ndarray, angles: np.ndarray, options, prec: str = "f",
          nthreads: int = 1) -> np.ndarray:
    """Apply a 2-D operator.  x: (B, H, W) image or (B, V, D) sinogram."""
    lib = _load()
    ang = np.ascontiguousarray(angles, dtype=np.float32)
    g = geom2_from_options(options, ang.size)
    dt = np.float32 if prec == "f" else np.float64
    ct = ctypes.c_float if prec == "f" else ctypes.c_double
    xin = np.ascontiguousarray(x, dtype=dt)
    batch = xin.shape[0]
    out = np.zeros(_out_shape2(g, op, batch), dtype=dt)
    fn = getattr(lib, f"ddo_{prec}_ddo_run2d")
    rc = fn(ctypes.byref(g), GEOM2[geom], OPS[op], _ptr(ang, ctypes.c_float), _ptr(xin, ct),
            _ptr(out, ct), batch, int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle run2d rejected geom={geom} op={op}")
    return out


def run3d(geom: str, op: str, x: np.ndarray, angles: np.ndarray, options,
          source_pos: np.ndarray | None = None, prec: str = "f", nthreads: int = 1) -> np.ndarray:
    """Apply a 3-D operator.  x: (B, Dep, H, W) volume or (B, V, Rows, Cols) sinogram."""
    lib = _load()
    ang = np.ascontiguousarray(angles, dtype=np.float32)
    g = geom3_from_options(options, ang.size, spiral=(geom == "spiral"))
    dt = np.float32 if prec == "f" else np.float64
    ct = ctypes.c_float if prec == "f" else ctypes.c_double
    xin = np.ascontiguousarray(x, dtype=dt)
    batch = xin.shape[0]
    if op in IMAGE_INPUT:
        shape = (batch, g.nv, g.nrow, g.ncol)
    else:
        shape = (batch, g.depth, g.height, g.width)
    out = np.zeros(shape, dtype=dt)
    sp = None
    if source_pos is not None:
        sp = np.ascontiguousarray(source_pos, dtype=np.float32)
    fn = getattr(lib, f"ddo_{prec}_ddo_run3d")
    rc = fn(ctypes.byref(g), GEOM3[geom], OPS[op], _ptr(ang, ctypes.c_float),
            _ptr(sp, ctypes.c_float) if sp is not None else None, _ptr(xin, ct), _ptr(out, ct),
            batch, int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle run3d rejected geom={geom} op={op}")
    return out


# margin of the start-index scan, in detector cells / pixels: some 20 to 50
# times the few-ulp differences between this FP32 restatement and the device
# code (fused multiply-adds, its own tan / atan), far below one cell
SCAN_MARGIN = 1e-3


def scan_hazards(geom: str, angles: np.ndarray, options, source_pos: np.ndarray | None = None,
                 margin: float = SCAN_MARGIN) -> np.ndarray:
    """Walk starts of deeprecon's CUDA kernels that could round to index -1.

    Returns, per view, how many (256-column block, image line) starts of the
    reference kernels lie within ``margin`` of a negative detector or pixel
    index on this geometry (ddoracle_body.h, ``ddo_scan2d`` / ``ddo_scan3d``).
    Only views with 0 are run on the reference kernels (``safe_views``)."""
    lib = _load()
    ang = np.ascontiguousarray(angles, dtype=np.float32)
    per = np.zeros(ang.size, np.int32)
    pv = _ptr(per, ctypes.c_int)
    if geom in GEOM2:
        g = geom2_from_options(options, ang.size)
        lib.ddo_f_ddo_scan2d(ctypes.byref(g), GEOM2[geom], _ptr(ang, ctypes.c_float), float(margin), pv)
        return per
    g = geom3_from_options(options, ang.size, spiral=(geom == "spiral"))
    sp = None if source_pos is None else np.ascontiguousarray(source_pos, dtype=np.float32)
    n = lib.ddo_f_ddo_scan3d(ctypes.byref(g), GEOM3[geom], _ptr(ang, ctypes.c_float),
                             _ptr(sp, ctypes.c_float) if sp is not None else None, float(margin), pv)
    if n < 0:
        raise ValueError("spiral scan needs source_pos")
    return per


def safe_views(geom: str, angles: np.ndarray, options, source_pos: np.ndarray | None = None) -> np.ndarray:
    """Indices of the views on which deeprecon's CUDA kernels start every walk
    at least ``SCAN_MARGIN`` away from a negative index."""
    return np.flatnonzero(scan_hazards(geom, angles, options, source_pos) == 0)


_REF_NAMES = {
    ("para", "proj"): "ProjParaDisCPU2d", ("para", "proj_t"): "ProjTransParaDisCPU2d",
    ("para", "bproj"): "BackProjParaDisCPU2d", ("para", "bproj_t"): "BackProjTransParaDisCPU2d",
}
for _g, _n in (("flat", "FanFlat"), ("arc", "FanArc")):
    _REF_NAMES.update({
        (_g, "proj"): f"Proj{_n}DisCPU2d", (_g, "proj_t"): f"ProjTrans{_n}DisCPU2d",
        (_g, "bproj"): f"BackProj{_n}DisCPU2d", (_g, "bproj_t"): f"BackProjTrans{_n}DisCPU2d",
        (_g, "bproj_w"): f"BackProjWeighted{_n}DisCPU2d",
        (_g, "bproj_tw"): f"BackProjTransWeighted{_n}DisCPU2d",
    })


def ref2d(geom: str, op: str, x: np.ndarray, angles: np.ndarray, options) -> np.ndarray:
    """Run deeprecon's own CPU code (threads chosen by the reference itself)."""
    lib = _load_ref()
    ang = np.ascontiguousarray(angles, dtype=np.float32)
    g = geom2_from_options(options, ang.size)
    xin = np.ascontiguousarray(x, dtype=np.float32)
    batch = xin.shape[0]
    out = np.zeros(_out_shape2(g, op, batch), dtype=np.float32)
    if op in IMAGE_INPUT:
        img, proj = xin, out
    else:
        img, proj = out, xin
    fn = getattr(lib, "ref_" + _REF_NAMES[(geom, op)])
    fptr = ctypes.POINTER(ctypes.c_float)
    fn.restype = None
    fn.argtypes = [fptr, fptr, fptr] + [ctypes.c_int] * 5 + [ctypes.c_float] * 8
    fn(_ptr(img, ctypes.c_float), _ptr(proj, ctypes.c_float), _ptr(ang, ctypes.c_float),
       batch, g.width, g.height, g.nv, g.nd, g.pix_x, g.pix_y, g.det_size, g.iso_source,
       g.source_detector, g.pix_xshift, g.pix_yshift, g.bin_shift)
    return out


def ref_sysmatrix(geom: str, angles: np.ndarray, options):
    """deeprecon's CPU COO system matrix: (rows, cols, vals)."""
    lib = _load_ref()
    ang = np.ascontiguousarray(angles, dtype=np.float32)
    g = geom2_from_options(options, ang.size)
    rows = ctypes.POINTER(ctypes.c_int64)()
    cols = ctypes.POINTER(ctypes.c_int64)()
    vals = ctypes.POINTER(ctypes.c_float)()
    n = lib.ref_sysmatrix(GEOM2[geom], _ptr(ang, ctypes.c_float), g.width, g.height, g.nv, g.nd,
                          g.pix_x, g.pix_y, g.det_size, g.iso_source, g.source_detector,
                          g.pix_xshift, g.pix_yshift, g.bin_shift, ctypes.byref(rows),
                          ctypes.byref(cols), ctypes.byref(vals))
    r = np.ctypeslib.as_array(rows, shape=(max(n, 1),))[:n].copy()
    c = np.ctypeslib.as_array(cols, shape=(max(n, 1),))[:n].copy()
    v = np.ctypeslib.as_array(vals, shape=(max(n, 1),))[:n].copy()
    for p in (rows, cols, vals):
        lib.ref_free(ctypes.cast(p, ctypes.c_void_p))
    return r, c, v

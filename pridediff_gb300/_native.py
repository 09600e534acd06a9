"""Build and load the native library ``libpridediff_dd.so`` (CUDA, sm_103a).

The library is the whole compute path: the Python layer only validates
arguments, allocates outputs / workspace with the torch caching allocator and
passes raw device pointers and the current CUDA stream through the C ABI
declared in ``include/pridediff_dd.h``.  There is no CPU fallback: if the
library is missing or a GPU is absent, every operator raises.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)
_CSRC = os.path.join(_PKG, "csrc")
_BUILD = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(_BUILD, "libpridediff_dd.so")
INCLUDE = os.path.join(_ROOT, "include")

# translation units of the library (compiled in parallel)
SOURCES = ["dd2d.cu", "dd2d_batch.cu", "dd2d_sysmat.cu", "dd3d.cu", "dd2d_noalloc.cu", "dd_fbp.cu"]

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH_FLAGS + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                           "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE]

_lock = threading.Lock()
_lib = None


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


# Build variants: the product library, and a test-only copy whose bounded
# waits give up at once (DD_WAIT_LIMIT=0) so that the timeout path -- skip the
# work, let the copies in flight land, record DD_ERR_TIMEOUT, return -- runs
# on a GPU without a fault or a hang.  The variant is never loaded by the
# package itself.
VARIANTS = {None: [], "waittest": ["-DDD_WAIT_LIMIT=0"]}


def lib_path(variant=None) -> str:
    return LIB_PATH if variant is None else os.path.join(_BUILD, variant, "libpridediff_dd.so")


def build(force: bool = False, verbose: bool = False, variant=None) -> str:
    """Compile every translation unit for sm_103a and link the shared library."""
    out_path = lib_path(variant)
    bdir = os.path.dirname(out_path)
    os.makedirs(bdir, exist_ok=True)
    srcs = [os.path.join(_CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(_CSRC, f) for f in os.listdir(_CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if not force and os.path.exists(out_path):
        lib_m = os.path.getmtime(out_path)
        if all(os.path.getmtime(d) <= lib_m for d in deps):
            return out_path
    nvcc = _nvcc()
    objs = [os.path.join(bdir, os.path.splitext(s)[0] + ".o") for s in SOURCES]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc, *NVCC_FLAGS, *VARIANTS[variant], "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = out_path + ".tmp"
    r = subprocess.run([nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs, "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, out_path)
    return out_path


class _Geom2d(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("num_det", ctypes.c_int)] + \
        [(n, ctypes.c_float) for n in ("pix_x", "pix_y", "det_size", "iso_source", "source_detector",
                                        "pix_xshift", "pix_yshift", "bin_shift")]


class _Instance2d(ctypes.Structure):
    _fields_ = [("geom", _Geom2d), ("num_view", ctypes.c_int), ("batch", ctypes.c_int)]


class _Tune2d(ctypes.Structure):
    _fields_ = [("ctas_per_sm", ctypes.c_int), ("lpt_order", ctypes.c_int), ("fwd_slices", ctypes.c_int),
                ("fwd_cluster", ctypes.c_int), ("items_cluster", ctypes.c_int), ("reserved", ctypes.c_int * 3)]


class _Geom3d(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("width", "height", "depth", "num_col", "num_row")] + \
        [(n, ctypes.c_float) for n in ("pix_x", "pix_y", "pix_z", "col_size", "row_size",
                                        "iso_source", "source_detector", "pix_xshift", "pix_yshift",
                                        "pix_zshift", "col_shift", "row_shift")]


Geom2d = _Geom2d
Geom3d = _Geom3d
Instance2d = _Instance2d
Tune2d = _Tune2d

# status codes (include/pridediff_dd.h)
DD_OK = 0
DD_ERR_INVALID_ARG = 1
DD_ERR_SIZE_OVERFLOW = 2
DD_ERR_WORKSPACE = 3
DD_ERR_LAUNCH = 4
DD_ERR_TIMEOUT = 5
DD_ERR_UNSUPPORTED = 6

SCAN2D = {"para": 0, "flat": 1, "arc": 2}
SCAN3D = {"cone_flat": 0, "cone_arc": 1, "spiral": 2}
OPS = {"proj": 0, "proj_t": 1, "bproj": 2, "bproj_t": 3, "bproj_w": 4, "bproj_tw": 5}


def _declare(lib):
    vp, sz, i, cp = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_char_p
    g2 = ctypes.POINTER(_Geom2d)
    lib.dd2d_workspace_bytes.restype = sz
    lib.dd2d_workspace_bytes.argtypes = [i, i, g2, i, i]
    lib.dd2d_apply.restype = i
    lib.dd2d_apply.argtypes = [i, i, g2, vp, vp, vp, i, i, vp, sz, vp]
    lib.dd2d_plan_bytes.restype = sz
    lib.dd2d_plan_bytes.argtypes = [i, g2, i]
    lib.dd2d_plan.restype = i
    lib.dd2d_plan.argtypes = [i, g2, vp, i, vp, sz, vp]
    lib.dd2d_apply_workspace_bytes.restype = sz
    lib.dd2d_apply_workspace_bytes.argtypes = [i, i, g2, i, i]
    lib.dd2d_apply_planned.restype = i
    lib.dd2d_apply_planned.argtypes = [i, i, g2, vp, vp, vp, i, i, vp, sz, vp]
    ip = ctypes.POINTER(_Instance2d)
    tp = ctypes.POINTER(_Tune2d)
    lib.dd2d_apply_planned_tuned.restype = i
    lib.dd2d_apply_planned_tuned.argtypes = [i, i, g2, vp, vp, vp, i, i, vp, sz, tp, vp]
    lib.dd2d_fwd_shape.restype = i
    lib.dd2d_fwd_shape.argtypes = [i, g2, tp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.dd2d_dc_workspace_bytes.restype = sz
    lib.dd2d_dc_workspace_bytes.argtypes = [i, g2, i, i]
    lib.dd2d_dc_step.restype = i
    lib.dd2d_dc_step.argtypes = [i, g2, vp, vp, vp, vp, ctypes.c_float, i, i, vp, sz, vp]
    lib.dd2d_batch_plan_bytes.restype = sz
    lib.dd2d_batch_plan_bytes.argtypes = [i, ip, i]
    lib.dd2d_batch_workspace_bytes.restype = sz
    lib.dd2d_batch_workspace_bytes.argtypes = [i, ip, i]
    lib.dd2d_batch_plan.restype = i
    lib.dd2d_batch_plan.argtypes = [i, ip, i, ctypes.POINTER(ctypes.c_void_p), vp, sz, tp, vp]
    lib.dd2d_batch_apply.restype = i
    lib.dd2d_batch_apply.argtypes = [i, i, ip, i, vp, vp, vp, vp, sz, tp, vp]
    lib.dd2d_batch_dc_step.restype = i
    lib.dd2d_batch_dc_step.argtypes = [i, ip, i, vp, vp, vp, ctypes.c_float, vp, sz, tp, vp]
    lib.dd2d_batch_status.restype = i
    lib.dd2d_batch_status.argtypes = [i, ip, i, vp, ctypes.POINTER(ctypes.c_int)]
    lib.dd2d_validate.restype = i
    lib.dd2d_validate.argtypes = [i, i, g2, i, i]
    lp = ctypes.POINTER(ctypes.c_longlong)
    lib.dd2d_sysmatrix_lines.restype = sz
    lib.dd2d_sysmatrix_lines.argtypes = [g2, i]
    lib.dd2d_sysmatrix_count.restype = i
    lib.dd2d_sysmatrix_count.argtypes = [i, g2, vp, i, vp, vp]
    lib.dd2d_sysmatrix_fill.restype = i
    lib.dd2d_sysmatrix_fill.argtypes = [i, g2, vp, i, vp, vp, vp, vp, vp]
    g3 = ctypes.POINTER(_Geom3d)
    lib.dd3d_validate.restype = i
    lib.dd3d_validate.argtypes = [i, i, g3, i, i]
    lib.dd3d_workspace_bytes.restype = sz
    lib.dd3d_workspace_bytes.argtypes = [i, i, g3, i, i]
    lib.dd3d_apply.restype = i
    lib.dd3d_apply.argtypes = [i, i, g3, vp, vp, vp, vp, i, i, vp, sz, vp]
    lib.dd3d_plan_bytes.restype = sz
    lib.dd3d_plan_bytes.argtypes = [i, g3, i]
    lib.dd3d_plan.restype = i
    lib.dd3d_plan.argtypes = [i, g3, vp, vp, i, vp, sz, vp]
    lib.dd3d_apply_workspace_bytes.restype = sz
    lib.dd3d_apply_workspace_bytes.argtypes = [i, i, g3, i, i]
    lib.dd3d_apply_planned.restype = i
    lib.dd3d_apply_planned.argtypes = [i, i, g3, vp, vp, vp, i, i, vp, sz, vp]
    lib.dd3d_dc_workspace_bytes.restype = sz
    lib.dd3d_dc_workspace_bytes.argtypes = [i, g3, i, i]
    lib.dd3d_dc_step.restype = i
    lib.dd3d_dc_step.argtypes = [i, g3, vp, vp, vp, vp, ctypes.c_float, i, i, vp, sz, vp]
    lib.dd_launch_count.restype = ctypes.c_ulonglong
    lib.dd_launch_count.argtypes = []
    lib.dd_profile_enable.restype = i
    lib.dd_profile_enable.argtypes = [i]
    lib.dd_profile_read.restype = i
    lib.dd_profile_read.argtypes = [i, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
    lib.dd_status_string.restype = cp
    lib.dd_status_string.argtypes = [i]
    lib.dd_version.restype = cp
    lib.dd_version.argtypes = []
    ip_ = ctypes.POINTER(ctypes.c_int)
    lib.dd2d_status.restype = i
    lib.dd2d_status.argtypes = [i, i, g2, i, i, vp, ip_]
    lib.dd2d_planned_status.restype = i
    lib.dd2d_planned_status.argtypes = [i, g2, i, i, vp, ip_]
    lib.dd3d_status.restype = i
    lib.dd3d_status.argtypes = [i, i, g3, i, i, vp, ip_]
    lib.dd3d_planned_status.restype = i
    lib.dd3d_planned_status.argtypes = [i, g3, i, i, vp, ip_]
    lib.dd_set_status_sink.restype = i
    lib.dd_set_status_sink.argtypes = [vp]
    lib.dd_noalloc_status.restype = i
    lib.dd_noalloc_status.argtypes = [ip_]
    lib.dd_fbp_filter.restype = i
    lib.dd_fbp_filter.argtypes = [vp, vp, vp, i, vp, ctypes.c_longlong, i, vp]


def load():
    """The loaded library; raises RuntimeError if it cannot be built or loaded."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                try:
                    build()
                except Exception as e:  # no nvcc: fail loudly, never fall back
                    raise RuntimeError(f"pridediff_gb300 native library unavailable: {e}") from e
            lib = ctypes.CDLL(LIB_PATH)
            _declare(lib)
            _lib = lib
        return _lib


def load_variant(variant: str):
    """A test-only build variant (see VARIANTS), built on first use."""
    path = build(variant=variant)
    lib = ctypes.CDLL(path)
    _declare(lib)
    return lib


def status_string(code: int) -> str:
    return load().dd_status_string(int(code)).decode()


def check(code: int, what: str) -> None:
    if code != DD_OK:
        raise RuntimeError(f"{what}: {status_string(code)} (status {code})")


def geom2d(options) -> _Geom2d:
    """dd_geom2d from the 11 entries of a projector2d options vector."""
    o = [float(x) for x in options]
    if len(o) != 11:
        raise RuntimeError("2-D options must have 11 entries (projector.py:113)")
    return _Geom2d(int(o[0]), int(o[1]), int(o[2]), *o[3:11])


def geom3d(options, spiral: bool = False) -> _Geom3d:
    o = [float(x) for x in options]
    if spiral:
        if len(o) != 16:
            raise RuntimeError("spiral options must have 16 entries (projector.py:460)")
        o = o[:14] + [0.0] + o[14:]
    elif len(o) != 17:
        raise RuntimeError("3-D options must have 17 entries (projector.py:286)")
    return _Geom3d(*(int(x) for x in o[:5]), *o[5:17])

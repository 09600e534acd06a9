import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "dd2d_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def sysmat_golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "sysmat_golden.npz"))


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


class _G2(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("num_det", ctypes.c_int)] + \
        [(n, ctypes.c_float) for n in ("pix_x", "pix_y", "det_size", "iso_source", "source_detector",
                                        "pix_xshift", "pix_yshift", "bin_shift")]


class HostModel:
    """ctypes wrapper of tests/native/dd_model2d.cpp (host model of the kernels)."""
    OPS = {"proj": 0, "proj_t": 1, "bproj": 2, "bproj_t": 3, "bproj_w": 4, "bproj_tw": 5}
    SCAN = {"para": 0, "flat": 1, "arc": 2}

    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        fp = ctypes.POINTER(ctypes.c_float)
        self.lib.model_apply2d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_G2), fp, fp, fp,
                                           ctypes.c_int, ctypes.c_int]
        self.lib.model_check_pieces.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_float)]

    def apply2d(self, geom, op, x, angles, opt):
        fp = ctypes.POINTER(ctypes.c_float)
        g = _G2(int(opt[0]), int(opt[1]), int(opt[2]), *[float(v) for v in opt[3:]])
        V = len(angles)
        B = x.shape[0]
        shape = (B, V, int(opt[2])) if op in ("proj", "bproj_t", "bproj_tw") else (B, int(opt[1]), int(opt[0]))
        out = np.zeros(shape, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        a = np.ascontiguousarray(angles, np.float32)
        rc = self.lib.model_apply2d(self.SCAN[geom], self.OPS[op], ctypes.byref(g), x.ctypes.data_as(fp),
                                    out.ctypes.data_as(fp), a.ctypes.data_as(fp), B, V)
        assert rc == 0
        return out

    def sysmatrix2d(self, geom, angles, opt):
        """(rows, cols, vals) of the system matrix through the kernels' line walk."""
        lp, fp = ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_float)
        f = self.lib.model_sysmatrix2d
        f.restype = ctypes.c_longlong
        f.argtypes = [ctypes.c_int, ctypes.POINTER(_G2), fp, ctypes.c_int, lp, lp, fp]
        g = _G2(int(opt[0]), int(opt[1]), int(opt[2]), *[float(v) for v in opt[3:]])
        a = np.ascontiguousarray(angles, np.float32)
        n = f(self.SCAN[geom], ctypes.byref(g), a.ctypes.data_as(fp), len(a), None, None, None)
        rows, cols, vals = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n, np.float32)
        f(self.SCAN[geom], ctypes.byref(g), a.ctypes.data_as(fp), len(a), rows.ctypes.data_as(lp),
          cols.ctypes.data_as(lp), vals.ctypes.data_as(fp))
        return rows, cols, vals

    def check_pieces(self, v0, pint, i0, nend):
        npc, fl, dev = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        bad = self.lib.model_check_pieces(ctypes.c_float(v0), ctypes.c_float(pint), i0, nend,
                                          ctypes.byref(npc), ctypes.byref(fl), ctypes.byref(dev))
        return bad, npc.value, fl.value, dev.value


@pytest.fixture(scope="session")
def host_model():
    src = os.path.join(ROOT, "tests", "native", "dd_model2d.cpp")
    outdir = os.path.join(ROOT, "tests", "native", "_build")
    os.makedirs(outdir, exist_ok=True)
    so = os.path.join(outdir, "libddmodel2d.so")
    hdrs = [os.path.join(ROOT, "pridediff_gb300", "csrc", f) for f in ("dd_geom.cuh", "dd_geom2d.cuh")]
    if not os.path.exists(so) or any(os.path.getmtime(p) > os.path.getmtime(so) for p in [src] + hdrs):
        r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", src,
                            "-o", so], capture_output=True, text=True)
        if r.returncode != 0:
            pytest.skip("host model does not compile here: " + r.stderr[-400:])
    return HostModel(so)


class _G3(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("width", "height", "depth", "num_col", "num_row")] + \
        [(n, ctypes.c_float) for n in ("pix_x", "pix_y", "pix_z", "col_size", "row_size", "iso_source",
                                        "source_detector", "pix_xshift", "pix_yshift", "pix_zshift",
                                        "col_shift", "row_shift")]


class HostModel3:
    """ctypes wrapper of tests/native/dd_model3d.cpp (host model of the 3-D kernels)."""
    OPS = {"proj": 0, "proj_t": 1, "bproj": 2, "bproj_t": 3, "bproj_w": 4, "bproj_tw": 5}
    SCAN = {"cone_flat": 0, "cone_arc": 1, "spiral": 2}

    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        fp = ctypes.POINTER(ctypes.c_float)
        self.lib.model_apply3d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_G3), fp, fp, fp, fp,
                                           ctypes.c_int, ctypes.c_int]

    def apply3d(self, geom, op, x, angles, opt, source_pos=None):
        fp = ctypes.POINTER(ctypes.c_float)
        o = [float(v) for v in opt]
        if geom == "spiral":
            o = o[:14] + [0.0] + o[14:]
        g = _G3(*[int(v) for v in o[:5]], *o[5:])
        V, B = len(angles), x.shape[0]
        shape = (B, V, g.num_row, g.num_col) if op in ("proj", "bproj_t", "bproj_tw") else \
            (B, g.depth, g.height, g.width)
        out = np.zeros(shape, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        a = np.ascontiguousarray(angles, np.float32)
        sp = None if source_pos is None else np.ascontiguousarray(source_pos, np.float32).ctypes.data_as(fp)
        rc = self.lib.model_apply3d(self.SCAN[geom], self.OPS[op], ctypes.byref(g), a.ctypes.data_as(fp), sp,
                                    x.ctypes.data_as(fp), out.ctypes.data_as(fp), B, V)
        assert rc == 0
        return out


@pytest.fixture(scope="session")
def host_model3():
    src = os.path.join(ROOT, "tests", "native", "dd_model3d.cpp")
    outdir = os.path.join(ROOT, "tests", "native", "_build")
    os.makedirs(outdir, exist_ok=True)
    so = os.path.join(outdir, "libddmodel3d.so")
    deps = [src] + [os.path.join(ROOT, "pridediff_gb300", "csrc", f)
                    for f in ("dd_geom.cuh", "dd_geom3d.cuh")]
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(d) for d in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", so],
                       check=True)
    return HostModel3(so)

"""Seeded 3-D test cases shared by the host-model (CPU) and GPU tests.

Each case is (geometry, options, angles, source_pos).  Options follow
deeprecon's projector3d / projectorsp packing (projector.py:286, :460):
cone (17): W, H, D, cols, rows, px, py, pz, col_size, row_size, SID, SDD,
           pix_xshift, pix_yshift, pix_zshift, col_shift, row_shift;
spiral (16): the same without pix_zshift.  Arc column sizes and shifts are
angles (projector.py:283-285).  The angle sets include views at exactly 45
and 135 degrees (the x/y branch boundary) and views that flip the detector.
"""
import numpy as np

OPS = ["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"]
IMAGE_IN = ("proj", "bproj_t", "bproj_tw")


def _angles(V, offset=0.05):
    a = (np.arange(V) * 2 * np.pi / V + offset).astype(np.float32)
    if V >= 8:
        a[1] = np.float32(np.pi / 4)
        a[2] = np.float32(3 * np.pi / 4)
    return a


def spiral_source(V, pitch, z0, drad=0.0, dang=0.0, daxial=0.0):
    sp = np.zeros((4, V), np.float32)
    sp[0] = (z0 + pitch * np.arange(V)).astype(np.float32)
    sp[1] = drad
    sp[2] = dang
    sp[3] = daxial
    return sp


def cases():
    out = {}
    out["cone_flat_small"] = ("cone_flat", np.array(
        [24, 20, 12, 40, 18, 1.3, 1.2, 1.1, 1.0, 1.0, 300.0, 600.0, 0.3, -0.2, 0.4, 0.7, 0.3], np.float32),
        _angles(10), None)
    out["cone_flat_blocks"] = ("cone_flat", np.array(   # 300 columns: two walk blocks
        [40, 40, 16, 300, 20, 1.0, 1.0, 1.0, 0.5, 1.0, 500.0, 1000.0, 0, 0, 0, 0, 0], np.float32),
        _angles(6), None)
    out["cone_arc_small"] = ("cone_arc", np.array(
        [24, 24, 12, 40, 18, 1.2, 1.2, 1.1, 1.5 / 600, 1.0, 300.0, 600.0, 0.2, 0.1, -0.3, 0.2 / 600, 0.2],
        np.float32), _angles(10), None)
    V = 12
    out["spiral_small"] = ("spiral", np.array(
        [24, 24, 16, 40, 8, 1.2, 1.2, 1.0, 1.6 / 600, 1.0, 300.0, 600.0, 0.1, 0.2, 0.3 / 600, 0.1], np.float32),
        _angles(V), spiral_source(V, 0.7, -4.0, 0.5, 0.001, 0.1))
    V = 16
    out["spiral_blocks"] = ("spiral", np.array(   # 270 columns, pitch: most views see part of the volume
        [32, 32, 24, 270, 8, 0.9, 0.9, 1.0, 0.6 / 600, 1.0, 400.0, 700.0, 0.0, 0.0, 0.0, 0.0], np.float32),
        _angles(V), spiral_source(V, 1.2, -9.0))
    return out


def inputs(case, batch=2, seed=0):
    geom, opt, ang, sp = case
    W, H, D, C, R = [int(v) for v in opt[:5]]
    rng = np.random.default_rng(seed)
    x = rng.random((batch, D, H, W)).astype(np.float32)
    y = rng.random((batch, len(ang), R, C)).astype(np.float32)
    return x, y

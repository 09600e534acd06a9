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


def ellipsoids(D, H, W, n, seed, scale=1.0):
    """Sum of n seeded random ellipsoids (intensity U[0, 1] x scale), rasterised
    at voxel centres in FP64 (the same bits on every host)."""
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.mgrid[0:D, 0:H, 0:W].astype(np.float64)
    vol = np.zeros((D, H, W))
    for _ in range(n):
        c = [rng.uniform(0.2, 0.8) * s for s in (D, H, W)]
        ax = [rng.uniform(0.05, 0.3) * s for s in (D, H, W)]
        vol[((zz - c[0]) / ax[0]) ** 2 + ((yy - c[1]) / ax[1]) ** 2 + ((xx - c[2]) / ax[2]) ** 2 <= 1] += \
            rng.uniform(0, 1)
    return (vol * scale).astype(np.float32)


def cone_256cube():
    """The cone-beam configuration: 256^3 at 1 mm, 512 x 384 detector of
    1 mm cells, SID 500 / SDD 1000, 360 views over 360 degrees."""
    opt = np.array([256, 256, 256, 512, 384, 1.0, 1.0, 1.0, 1.0, 1.0, 500.0, 1000.0, 0, 0, 0, 0, 0], np.float32)
    return opt, (np.arange(360) * 2 * np.pi / 360).astype(np.float32)


def spiral_512x128():
    """The spiral configuration: 512 x 512 x 128 at 0.66 x 0.66 x 1 mm, 64 x 736
    arc detector (1.2858 mm columns at SDD 1085.6, 1 mm rows), 1152 views per
    turn, pitch 1, 3 turns, trajectory centred on the volume."""
    V = 3456
    p = 1.0 * 64 * 1.0 * 595.0 / 1085.6 / 1152
    opt = np.array([512, 512, 128, 736, 64, 0.66, 0.66, 1.0, 1.2858 / 1085.6, 1.0, 595.0, 1085.6, 0.0, 0.0,
                    0.0, 0.0], np.float32)
    ang = (np.arange(V) * 2 * np.pi / 1152).astype(np.float32)
    return opt, ang, spiral_source(V, p, -p * (V - 1) / 2)


# view subsets of the full configurations kept as golden vectors, with the
# strides that subsample their outputs (full outputs would be tens of MB)
CONE_VIEWS = np.array([0, 45, 100, 271])
SPIRAL_VIEWS = np.array([0, 700, 1500, 1728, 2600, 3455])
CONE_SINO_STRIDE = (slice(None), slice(None), slice(None, None, 4), slice(None))      # (B, V, R, C)
CONE_VOL_STRIDE = (slice(None), slice(None, None, 8), slice(None, None, 4), slice(None, None, 4))
SPIRAL_SINO_STRIDE = (slice(None), slice(None), slice(None, None, 2), slice(None))
SPIRAL_VOL_STRIDE = (slice(None), slice(None, None, 4), slice(None, None, 8), slice(None, None, 8))

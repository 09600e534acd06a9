"""The FBP pixel weight as the 2-D kernels evaluate it, against the
reference's FP32 sequence (FanFlatDisCPU2d.cpp:693, FanArcDisCPU2d.cpp:703).

Flat detector: the reference computes d = (sx px + sy py) / r, t = r - d,
w = r^2 / t^2 (two divisions); the kernels compute (r^2 / (r^2 - s.p))^2 with
one division.  Arc detector: 1 / |s - p|^2.  Both are emulated here in FP32
(numpy) over the fan geometries the tests and the benchmark use: the two
sequences differ by at most 7.2 ulp of FP32 (4.3e-7 relative; the kernels'
fast division adds at most 2 ulp on top of the correctly rounded one
emulated here), 20x inside the operators' 1e-5 parity bound.
"""
import numpy as np
import pytest

f32 = np.float32


def _grid(r, half, n=97):
    ang = np.linspace(0, 2 * np.pi, 64, endpoint=False)
    sx, sy = (r * np.cos(ang)).astype(f32), (r * np.sin(ang)).astype(f32)
    c = np.linspace(-half, half, n).astype(f32)
    px, py = np.meshgrid(c, c)
    return sx[:, None, None], sy[:, None, None], px[None].astype(f32), py[None].astype(f32)


def _flat_reference(sx, sy, px, py, r):
    d = (sx * px + sy * py) / r              # FP32 throughout, no FMA
    t = r - d
    return (r * r) / (t * t)


def _flat_kernel(sx, sy, px, py, r):
    r2 = r * r
    q = r2 - (sx * px + sy * py).astype(f32)
    t = r2 / q
    return t * t


@pytest.mark.parametrize("r,half", [(595.0, 169.0), (500.0, 128.0), (1000.0, 400.0)])
def test_flat_weight_within_a_few_ulp_of_the_reference(r, half):
    sx, sy, px, py = _grid(f32(r), half)
    ref = _flat_reference(sx, sy, px, py, f32(r)).astype(np.float64)
    got = _flat_kernel(sx, sy, px, py, f32(r)).astype(np.float64)
    rel = np.abs(got - ref) / ref
    assert rel.max() <= 10 * 2.0 ** -24, rel.max()


@pytest.mark.parametrize("r,half", [(595.0, 169.0), (500.0, 128.0)])
def test_arc_weight_is_the_reciprocal_squared_distance(r, half):
    sx, sy, px, py = _grid(f32(r), half)
    a, b = sx - px, sy - py
    ref = (f32(1.0) / (a * a + b * b)).astype(np.float64)
    exact = 1.0 / ((a.astype(np.float64)) ** 2 + (b.astype(np.float64)) ** 2)
    assert (np.abs(ref - exact) / exact).max() <= 4 * 2.0 ** -24

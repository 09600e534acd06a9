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


@pytest.mark.gpu
@pytest.mark.parametrize("scan", ["flat", "arc"])
def test_gpu_kernel_weight_against_fp64(scan):
    """The weight as the CUDA kernels apply it: for one view and a sinogram of
    ones, BackProjWeighted / BackProj at a pixel is that pixel's FBP weight
    (flat: r^2 / (r - s.p / r)^2; arc: 1 / |s - p|^2, which the reference
    divides by), up to the rounding of the two sums.  Compared with the FP64
    formula at the FP32 source and pixel-centre coordinates the kernels use."""
    import torch
    from pridediff_gb300 import radontorch as RT
    W = H = 64
    pix, R, SDD, D = 2.6, 595.0, 1085.6, 200
    det = 1.2858 / SDD if scan == "arc" else 1.2858
    opt = torch.tensor([W, H, D, pix, pix, det, R, SDD, 0.0, 0.0, 0.0], dtype=torch.float32)
    name = "FanFlat" if scan == "flat" else "FanArc"
    worst = 0.0
    for view in (0.3, 1.2, 2.9, 4.4, 5.95):
        ang = torch.tensor([view], dtype=torch.float32, device="cuda")
        ones = torch.ones((1, 1, 1, D), device="cuda")
        bp = getattr(RT, f"BackProj{name}Dis2d")(ones, opt, ang)[0, 0].double().cpu().numpy()
        bpw = getattr(RT, f"BackProjWeighted{name}Dis2d")(ones, opt, ang)[0, 0].double().cpu().numpy()
        v32 = np.float32(view)
        s, c = f32(np.sin(np.float64(v32))), f32(np.cos(np.float64(v32)))
        sx, sy = float(f32(-s * f32(R))), float(f32(c * f32(R)))
        cols = (np.arange(W) + 0.5) * pix - W / 2 * pix
        rows = H / 2 * pix - (np.arange(H) + 0.5) * pix
        px = cols.astype(f32).astype(np.float64)[None, :]
        py = rows.astype(f32).astype(np.float64)[:, None]
        if scan == "flat":
            d = (sx * px + sy * py) / R
            w = R * R / (R - d) ** 2
        else:
            w = 1.0 / ((sx - px) ** 2 + (sy - py) ** 2)
        m = bp > 1e-3 * bp.max()
        rel = np.abs(bpw[m] / bp[m] / w[m] - 1.0)
        worst = max(worst, float(rel.max()))
    print(f"{scan}: FBP weight as applied by the kernels vs FP64: {worst:.2e} relative")
    assert worst <= 16 * 2.0 ** -24

"""Filtered back-projection (deeprecon/torch/projector/projector.py:192-213,
368-390, 554-563) against deeprecon's own filtered_backprojection.

The fixtures (tests/golden/fbp_golden.npz, made by make_golden.py --fbp) hold
the reference's result for fan-flat (ramp), fan-arc (Shepp-Logan) and
parallel beams (ramp, redundant=False), and its filter taps and cosine
weights.  CPU tests pin the taps and weights bit for bit and check the
oracle's composition; GPU tests run the fused weight + filter kernel and the
weighted back-projection through projector2d / projector3d.
"""
import os

import numpy as np
import pytest
import torch

from conftest import ROOT, rel_l2

GOLDEN = os.path.join(ROOT, "tests", "golden", "fbp_golden.npz")
CASES = {"flat_fbp": ("flat", "ramp", True), "arc_fbp": ("arc", "sheeplogan", True),
         "para_fbp": ("para", "ramp", False)}


@pytest.fixture(scope="module")
def fbp_golden():
    return np.load(GOLDEN)


def _projector(gold, name):
    from pridediff_gb300.projector import projector2d
    geom, ftype, _ = CASES[name]
    c = [float(v) for v in gold[f"{name}/ctor"]]   # the reference constructor's arguments
    return projector2d((int(c[0]), int(c[1])), int(c[2]), (c[3], c[4]), c[5], c[6], c[7], (c[8], c[9]), c[10],
                       scan_type=geom, filter_type=ftype)


def _correlate(x, w, taps):
    """conv2d(x * w, taps, padding=D - 1) along the last axis, in float64."""
    D = x.shape[-1]
    xw = (x.astype(np.float32) * w.astype(np.float32)).astype(np.float64)
    T = np.empty((D, D))
    n = np.arange(D)
    for k in range(D):
        T[:, k] = taps[n - k + D - 1]
    return xw @ T


@pytest.mark.parametrize("name", sorted(CASES))
def test_taps_and_weights_match_reference(fbp_golden, name):
    """Filter taps and cosine weights equal to deeprecon's (fixtures made on an
    x86-64 host).  The weights come from torch's cos / atan: another host's
    math library may round a few of them one ulp apart."""
    import platform
    prj = _projector(fbp_golden, name)
    assert np.array_equal(prj.filter.detach().numpy().reshape(-1), fbp_golden[f"{name}/filter"])
    if platform.machine() in ("x86_64", "AMD64"):
        assert np.array_equal(prj.weight.detach().numpy(), fbp_golden[f"{name}/weight"])
    else:
        np.testing.assert_array_max_ulp(prj.weight.detach().numpy(), fbp_golden[f"{name}/weight"], maxulp=1)
    for other in ("ramp", "sheeplogan"):
        assert np.array_equal(prj.filter_generate(other).numpy().reshape(-1), fbp_golden[f"{name}/taps_{other}"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_fbp_matches_reference(fbp_golden, name):
    import oracle
    geom, _, redundant = CASES[name]
    sino, ang = fbp_golden[f"{name}/sino"], fbp_golden[f"{name}/angles"]
    filt = _correlate(sino, fbp_golden[f"{name}/weight"], fbp_golden[f"{name}/filter"].astype(np.float64))
    # parallel beams back-project with the plain DD-BP (projector.py:49)
    op = "bproj" if geom == "para" else "bproj_w"
    # FP32, as the reference computes: the filtered arc sinogram alternates in
    # sign at large magnitude, and the FP32 back-projection (the reference's
    # too) sits 2e-5 from an FP64 one, while the two FP32 results agree to 2e-7
    rec = oracle.run2d(geom, op, filt.astype(np.float32), ang, fbp_golden[f"{name}/options"], prec="f")
    scale = np.float32(abs(ang[-1] - ang[0])) / np.float32(len(ang) - 1)
    rec = rec * scale / (2.0 if redundant else 1.0)
    assert rel_l2(rec, fbp_golden[f"{name}/fbp"]) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_fbp_matches_reference(fbp_golden, name):
    _, _, redundant = CASES[name]
    prj = _projector(fbp_golden, name).cuda()
    sino = torch.from_numpy(fbp_golden[f"{name}/sino"])[:, None].cuda()
    ang = torch.from_numpy(fbp_golden[f"{name}/angles"]).cuda()
    rec = prj.filtered_backprojection(sino, ang, redundant=redundant)
    assert rel_l2(rec[:, 0].cpu().numpy(), fbp_golden[f"{name}/fbp"]) <= 1e-5


def _filter(x, w, taps):
    from pridediff_gb300 import fbp
    return fbp.FbpFilter.apply(x, w, taps)


@pytest.mark.gpu
@pytest.mark.parametrize("rows,D,wrows", [(1440, 736, 1), (7, 1, 1), (33, 5, 1), (64, 97, 8), (4, 2048, 2)])
def test_gpu_filter_kernel_against_fp64(rows, D, wrows):
    g = torch.Generator().manual_seed(rows * 31 + D)
    x = torch.randn(rows, D, generator=g)
    w = torch.rand(wrows, D, generator=g) + 0.5
    taps = torch.randn(2 * D - 1, generator=g)   # not symmetric
    out = _filter(x.cuda(), w.cuda(), taps.cuda()).cpu().numpy()
    wr = w.numpy()[np.arange(rows) % wrows]   # row i takes weight row i % wrows
    ref = _correlate(x.numpy(), wr, taps.numpy().astype(np.float64))
    assert rel_l2(out, ref) <= 1e-6


@pytest.mark.gpu
def test_gpu_filter_backward_is_the_transpose():
    g = torch.Generator().manual_seed(5)
    rows, D = 24, 61
    x = torch.randn(rows, D, generator=g).cuda().requires_grad_(True)
    w = (torch.rand(1, D, generator=g) + 0.5).cuda()
    taps = torch.randn(2 * D - 1, generator=g).cuda()
    y = torch.randn(rows, D, generator=g).cuda()
    out = _filter(x, w, taps)
    (out * y).sum().backward()
    lhs = float((out.detach().double() * y.double()).sum())
    rhs = float((x.detach().double() * x.grad.double()).sum())
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


@pytest.mark.gpu
def test_gpu_cone_fbp_matches_the_composition():
    from pridediff_gb300.projector import projector3d
    prj = projector3d((24, 20, 12), (40, 18), 1.0, (1.0, 1.0), 300.0, 600.0, scan_type="flat").cuda()
    g = torch.Generator().manual_seed(9)
    ang = (torch.arange(30, dtype=torch.float32) * (2 * np.pi / 30)).cuda()
    sino = torch.rand(2, 1, 30, 18, 40, generator=g).cuda()
    rec = prj.filtered_backprojection(sino, ang)
    w, taps = prj.weight.double(), prj.filter.double()
    filt = torch.nn.functional.conv3d(sino.double() * w, taps, padding=(0, 0, 39)).float()
    ref = prj.backprojection_w(filt, ang) * (ang[-1] - ang[0]).abs() / (ang.numel() - 1) / 2
    assert rel_l2(rec.cpu().numpy(), ref.cpu().numpy()) <= 1e-5


@pytest.mark.gpu
def test_gpu_trainable_filter_gets_a_gradient(fbp_golden):
    from pridediff_gb300.projector import projector2d
    prj = projector2d((32, 32), 40, 1.0, 1.0, 500.0, 1000.0, scan_type="flat", trainable=True).cuda()
    ang = (torch.arange(36, dtype=torch.float32) * (2 * np.pi / 36)).cuda()
    sino = torch.rand(1, 1, 36, 40, generator=torch.Generator().manual_seed(3)).cuda()
    rec = prj.filtered_backprojection(sino, ang)
    rec.square().sum().backward()
    assert prj.filter.grad is not None and torch.isfinite(prj.filter.grad).all()
    assert prj.weight.grad is not None and float(prj.weight.grad.abs().sum()) > 0

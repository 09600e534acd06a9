"""GPU tests of the uneven persistent batch and the fused / graph-captured
data-consistency step."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FAN = dict(pix=0.66, det=1.2858, sid=595.0, sdd=1085.6)


def _instances(seed, n, scan="flat"):
    """Uneven instances drawn like the reference's batched configuration:
    image from {256,384,512}^2, views from {360,576,720}, dets from {368,512,736}."""
    import pridediff_gb300 as P
    rng = np.random.default_rng(seed)
    projs, angs, batch = [], [], []
    for i in range(n):
        size = int(rng.choice([256, 384, 512]))
        V = int(rng.choice([360, 576, 720]))
        D = int(rng.choice([368, 512, 736]))
        det = FAN["det"] if scan != "arc" else FAN["det"]
        projs.append(P.projector2d(size, D, FAN["pix"], det, FAN["sid"], FAN["sdd"], scan_type=scan).cuda())
        angs.append(torch.arange(V, dtype=torch.float32, device="cuda") * (2 * np.pi / V))
        batch.append(int(rng.integers(1, 3)))
    return projs, angs, batch


def _rand_images(projs, batch, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return [torch.rand((b, 1, p.image_size[1], p.image_size[0]), device="cuda", generator=g) * 0.04
            for p, b in zip(projs, batch)]


@pytest.mark.parametrize("scan", ["flat", "arc", "para"])
def test_batched_forward_and_adjoint_equal_per_instance(scan):
    from pridediff_gb300.batch import UnevenBatch2d
    projs, angs, batch = _instances(1, 5, scan)
    ub = UnevenBatch2d(projs, angs, batch)
    xs = _rand_images(projs, batch, 2)
    ys = ub.unpack_sinos(ub.forward(ub.pack(xs)))
    # the single-geometry forward sums a view's lines as two interleaved
    # halves (one per CTA of a cluster), the persistent one in one sequence:
    # FP32 rounding apart; the adjoints are the same computation, bit for bit
    for p, a, x, y in zip(projs, angs, xs, ys):
        assert rel_l2(y.cpu().numpy(), p.projection(x, a).cpu().numpy()) <= 1e-6
    g = torch.Generator(device="cuda").manual_seed(3)
    rs = [torch.randn(s, device="cuda", generator=g) for s in ub.sino_shapes]
    bs = ub.unpack_images(ub.adjoint(ub.pack(rs)))
    for p, a, r, b in zip(projs, angs, rs, bs):
        assert torch.equal(b, p.projection_t(r, a))
    assert ub.device_status() == 0


def test_batched_autograd_and_tuning_do_not_change_results():
    from pridediff_gb300.batch import UnevenBatch2d
    projs, angs, batch = _instances(4, 4)
    ub = UnevenBatch2d(projs, angs, batch)
    x = ub.pack(_rand_images(projs, batch, 5)).requires_grad_(True)
    y = ub.project(x)
    w = torch.randn_like(y)
    (y * w).sum().backward()
    ref_grad = ub.adjoint(w)
    assert torch.equal(x.grad, ref_grad)
    y1 = ub.forward(x.detach())
    for cfg in ({"ctas_per_sm": 1, "lpt_order": 0}, {"ctas_per_sm": 3, "lpt_order": 1}):
        ub.set_tune(cfg)
        assert torch.equal(ub.forward(x.detach()), y1)


def test_fused_dc_step_matches_separate_operators():
    import pridediff_gb300 as P
    from pridediff_gb300 import dc
    proj = P.projector2d(256, 368, 1.32, 2.5716, 595.0, 1085.6).cuda()
    ang = torch.arange(360, dtype=torch.float32, device="cuda") * (2 * np.pi / 360)
    x = torch.rand((3, 1, 256, 256), device="cuda") * 0.04
    y = proj.projection(torch.rand_like(x) * 0.04, ang)
    eta = 1e-6
    expect = x - eta * proj.projection_t(proj.projection(x, ang) - y, ang)
    got = dc.dc_step(proj, x.clone(), y, ang, eta)
    assert rel_l2(got.cpu().numpy(), expect.cpu().numpy()) <= 1e-6
    r = dc.residual(proj, x, y, ang)
    assert torch.equal(r, proj.projection(x, ang) - y)


def test_dc_loss_gradient_is_the_exact_adjoint():
    import pridediff_gb300 as P
    from pridediff_gb300 import dc
    proj = P.projector2d(128, 184, 2.64, 5.1432, 595.0, 1085.6).cuda()
    ang = torch.arange(180, dtype=torch.float32, device="cuda") * (2 * np.pi / 180)
    y = proj.projection(torch.rand((2, 1, 128, 128), device="cuda"), ang)
    x = torch.rand((2, 1, 128, 128), device="cuda").requires_grad_(True)
    loss = dc.dc_loss(proj, x, y, ang)
    loss.backward()
    with torch.no_grad():
        r = proj.projection(x, ang) - y
        ref_loss = (r.double() ** 2).sum()
        ref_grad = 2 * proj.projection_t(r, ang)
    assert abs(loss.item() - ref_loss.item()) <= 1e-6 * ref_loss.item()
    assert rel_l2(x.grad.cpu().numpy(), ref_grad.cpu().numpy()) <= 1e-6


def test_graph_captured_dc_loop_equals_eager():
    from pridediff_gb300.batch import UnevenBatch2d
    projs, angs, batch = _instances(7, 6)
    ub = UnevenBatch2d(projs, angs, batch)
    x0 = ub.pack(_rand_images(projs, batch, 8))
    y = ub.forward(ub.pack(_rand_images(projs, batch, 9)))
    eta = 1e-7
    xe = x0.clone()
    for _ in range(5):
        ub.dc_step(xe, y, eta)
    xg = x0.clone()
    g = ub.dc_graph(xg, y, eta, 5)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(xg, xe)
    # the eager per-instance update with separate operators agrees to rounding
    xs = [t.clone() for t in ub.unpack_images(x0.clone())]
    ys = ub.unpack_sinos(y)
    for _ in range(5):
        xs = [x - eta * p.projection_t(p.projection(x, a) - yy, a) for p, a, x, yy in zip(projs, angs, xs, ys)]
    assert rel_l2(ub.pack(xs).cpu().numpy(), xe.cpu().numpy()) <= 1e-5


def test_config3_uneven_24_instances_50_captured_steps():
    """The reference's batched configuration: 24 uneven fan-flat instances,
    50 graph-captured steps of x <- x - 1e-3 A^T (A x - y).  With eta = 1e-3
    the iteration is unstable (lambda_max(A^T A) ~ 1e5), so values are checked
    on the first steps of a stable variant and the captured loop is checked to
    run to completion with the device status clear."""
    from pridediff_gb300.batch import UnevenBatch2d
    projs, angs, _ = _instances(2024, 24)
    ub = UnevenBatch2d(projs, angs, [1] * 24)
    x0 = ub.pack(_rand_images(projs, [1] * 24, 10))
    y = ub.forward(ub.pack(_rand_images(projs, [1] * 24, 11)))
    xs = x0.clone()
    g = ub.dc_graph(xs, y, 1e-3, 50)
    g.replay()
    torch.cuda.synchronize()
    assert ub.device_status() == 0
    # stable variant: eta well below 1 / lambda_max; compare 3 steps to separate ops
    eta = 1e-7
    xc = x0.clone()
    for _ in range(3):
        ub.dc_step(xc, y, eta)
    parts = [t.clone() for t in ub.unpack_images(x0.clone())]
    ys = ub.unpack_sinos(y)
    for _ in range(3):
        parts = [x - eta * p.projection_t(p.projection(x, a) - yy, a) for p, a, x, yy in zip(projs, angs, parts, ys)]
    assert rel_l2(ub.pack(parts).cpu().numpy(), xc.cpu().numpy()) <= 1e-5


def test_dc_step_size_against_power_iteration():
    """lambda_max(A^T A) of the 512^2 fan-flat geometry (720 views, 736
    detectors) by power iteration, and what it means for the batched
    configuration's step x <- x - eta A^T (A x - y): with eta below
    2 / lambda_max the residual falls every step, with eta = 1e-3 (the
    configuration's value) it grows."""
    import pridediff_gb300 as P
    proj = P.projector2d(512, 736, 0.66, 1.2858, 595.0, 1085.6, scan_type="flat").cuda()
    ang = torch.arange(720, dtype=torch.float32, device="cuda") * (2 * np.pi / 720)
    g = torch.Generator(device="cuda").manual_seed(9)
    v = torch.rand((1, 1, 512, 512), device="cuda", generator=g)
    lam = 0.0
    for _ in range(30):
        w = proj.projection_t(proj.projection(v, ang), ang)
        lam = float((w.double() * v.double()).sum() / (v.double() ** 2).sum())
        v = w / w.norm()
    print(f"lambda_max(A^T A) ~ {lam:.4e} (512^2, 720 views, 736 dets)")
    assert 1e4 < lam < 1e6
    x_true = torch.rand((1, 1, 512, 512), device="cuda", generator=g) * 0.04
    y = proj.projection(x_true, ang)

    def residuals(eta, steps):
        x = torch.zeros_like(x_true)
        out = []
        for _ in range(steps):
            r = proj.projection(x, ang) - y
            out.append(float(r.double().norm()))
            x = x - eta * proj.projection_t(r, ang)
        return out

    stable = residuals(1.0 / lam, 6)
    assert all(b < a for a, b in zip(stable, stable[1:]))
    unstable = residuals(1e-3, 6)
    assert unstable[-1] > 10 * unstable[0]


def test_uneven_24_instance_configuration_matches_reference_cpu(oracle_mod):
    """Every instance of the 24-instance uneven configuration (image sizes
    {256,384,512}^2, views {360,576,720}, detectors {368,512,736}; the draw
    bench.py times), forward and exact adjoint through the persistent batch,
    against the FP32 oracle (bit-exact with deeprecon's CPU path) at 1e-5."""
    import bench
    from pridediff_gb300.batch import UnevenBatch2d
    dev = torch.device("cuda", 0)
    projs, angs, imgs, _ = bench.uneven_instances(dev)
    ub = UnevenBatch2d(projs, angs)
    ys = ub.unpack_sinos(ub.forward(ub.pack(imgs)))
    g = torch.Generator(device="cuda").manual_seed(9)
    rs = [torch.randn(s, device="cuda", generator=g) for s in ub.sino_shapes]
    bs = ub.unpack_images(ub.adjoint(ub.pack(rs)))
    worst = 0.0
    for p, a, x, y, r, b in zip(projs, angs, imgs, ys, rs, bs):
        opt = p.options.cpu().numpy()
        ang = a.cpu().numpy()
        ef = rel_l2(y[:, 0].cpu().numpy(), oracle_mod.run2d("flat", "proj", x[:, 0].cpu().numpy(), ang, opt, "f", 16))
        ea = rel_l2(b[:, 0].cpu().numpy(), oracle_mod.run2d("flat", "proj_t", r[:, 0].cpu().numpy(), ang, opt, "f", 16))
        worst = max(worst, ef, ea)
        assert ef <= 1e-5 and ea <= 1e-5, (p.image_size, a.numel(), opt[2], ef, ea)
    print(f"24 uneven instances: worst rel-L2 vs reference CPU {worst:.2e}")


def test_instances_with_one_geometry_are_merged_without_changing_results():
    """Instances with the same geometry and angles become one multi-slice
    instance; every slice's forward and adjoint stay bit-identical."""
    import pridediff_gb300 as P
    from pridediff_gb300.batch import UnevenBatch2d
    sizes = [(256, 360, 368), (384, 576, 512), (256, 360, 368), (512, 360, 368), (384, 576, 512), (256, 360, 368)]
    projs = [P.projector2d(n, D, FAN["pix"], FAN["det"], FAN["sid"], FAN["sdd"], scan_type="flat").cuda()
             for n, _, D in sizes]
    angs = [torch.arange(V, dtype=torch.float32, device="cuda") * (2 * np.pi / V) for _, V, _ in sizes]
    batch = [1, 2, 1, 1, 1, 2]
    merged = UnevenBatch2d(projs, angs, batch)
    plain = UnevenBatch2d(projs, angs, batch, group=False)
    assert merged.n == 3 and plain.n == 6
    assert merged.groups == [[0, 2, 5], [1, 4], [3]]
    xs = _rand_images(projs, batch, 21)
    fm = merged.unpack_sinos(merged.forward(merged.pack(xs)))
    fp = plain.unpack_sinos(plain.forward(plain.pack(xs)))
    for a, b in zip(fm, fp):
        assert torch.equal(a, b)
    g = torch.Generator(device="cuda").manual_seed(22)
    rs = [torch.randn(s, device="cuda", generator=g) for s in plain.sino_shapes]
    am = merged.unpack_images(merged.adjoint(merged.pack(rs)))
    ap = plain.unpack_images(plain.adjoint(plain.pack(rs)))
    for a, b in zip(am, ap):
        assert torch.equal(a, b)

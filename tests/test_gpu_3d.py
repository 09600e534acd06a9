"""GPU parity of the 3-D operators (cone-flat, cone-arc, spiral) through the
radontorch drop-in and the C ABI.

deeprecon has no CPU path for 3-D (RadonTorch.cpp:604): its CUDA kernels are
the reference.  tests/golden/dd3d_golden.npz holds their outputs on the
small cases of cases3d.py and on view subsets of the full cone-beam and
spiral configurations (made by tests/golden/make_golden.py --cuda3d, which
runs the reference kernels compiled unmodified; test_gpu_refcuda.py compares
against those kernels directly where they are built).  Bars: rel-L2 <= 1e-5
against the reference's outputs; <= 5e-5 against the FP32 oracle, which
rounds its trigonometry correctly where the reference's device code and the
kernels here call CUDA's single-precision functions (the error against the
FP64 oracle is printed); dot-product adjointness <= 1e-6 with FP64
accumulation; bit-identical repeated runs.
"""
import numpy as np
import pytest
import torch

import cases3d
from cases3d import spiral_source
from conftest import rel_l2

pytestmark = pytest.mark.gpu

CASES = cases3d.cases()
GEO = {"cone_flat": "ConeFlat", "cone_arc": "ConeArc", "spiral": "Spiral"}
NAMES = {"proj": "Proj{}Dis3d", "proj_t": "ProjTrans{}Dis3d", "bproj": "BackProj{}Dis3d",
         "bproj_t": "BackProjTrans{}Dis3d", "bproj_w": "BackProjWeighted{}Dis3d",
         "bproj_tw": "BackProjTransWeighted{}Dis3d"}


def run(geom, op, x, angles, opt, sp=None):
    from pridediff_gb300 import radontorch
    fn = getattr(radontorch, NAMES[op].format(GEO[geom]))
    xt = torch.from_numpy(np.ascontiguousarray(x)[:, None]).cuda()
    at = torch.from_numpy(np.ascontiguousarray(angles, np.float32)).cuda()
    ot = torch.tensor(np.asarray(opt, np.float32))
    if geom == "spiral":
        out = fn(xt, ot, at, torch.from_numpy(np.ascontiguousarray(sp, np.float32)).cuda())
    else:
        out = fn(xt, ot, at)
    torch.cuda.synchronize()
    return out[:, 0].cpu().numpy()


@pytest.fixture(scope="module")
def golden3d():
    import os
    from conftest import ROOT
    return np.load(os.path.join(ROOT, "tests", "golden", "dd3d_golden.npz"))


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("op", cases3d.OPS)
def test_gpu_matches_reference_golden(golden3d, oracle_mod, name, op):
    geom, opt, ang, sp = CASES[name]
    x, y = cases3d.inputs(CASES[name], batch=1, seed=31)
    inp = x if op in cases3d.IMAGE_IN else y
    out = run(geom, op, inp, ang, opt, sp)
    e = rel_l2(out, golden3d[f"{name}/{op}/ref"])
    e64 = rel_l2(out, oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="d", nthreads=8))
    print(f"{name} {op}: rel-L2 vs reference CUDA outputs {e:.2e}, vs FP64 oracle {e64:.2e}")
    assert e <= 1e-5


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("op", cases3d.OPS)
def test_gpu_close_to_oracle(oracle_mod, name, op):
    geom, opt, ang, sp = CASES[name]
    x, y = cases3d.inputs(CASES[name], batch=3, seed=11)
    inp = x if op in cases3d.IMAGE_IN else y
    out = run(geom, op, inp, ang, opt, sp)
    ref = oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="f", nthreads=8)
    r64 = oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="d", nthreads=8)
    e32, e64 = rel_l2(out, ref), rel_l2(out, r64)
    print(f"{name} {op}: rel-L2 vs FP32 oracle {e32:.2e}, vs FP64 {e64:.2e}")
    assert e32 <= 5e-5


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_pairs_are_adjoint(name):
    geom, opt, ang, sp = CASES[name]
    x, y = cases3d.inputs(CASES[name], batch=2, seed=13)
    for fwd, adj in (("proj", "proj_t"), ("bproj_t", "bproj"), ("bproj_tw", "bproj_w")):
        ax = run(geom, fwd, x, ang, opt, sp).astype(np.float64)
        aty = run(geom, adj, y, ang, opt, sp).astype(np.float64)
        lhs, rhs = float((ax * y).sum()), float((x * aty).sum())
        print(f"{name} {fwd}/{adj}: dot rel {abs(lhs - rhs) / abs(lhs):.2e}")
        assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


def test_gpu_runs_are_deterministic():
    geom, opt, ang, sp = CASES["spiral_blocks"]
    x, y = cases3d.inputs(CASES["spiral_blocks"], batch=2, seed=17)
    for op, inp in (("proj", x), ("proj_t", y)):
        a = run(geom, op, inp, ang, opt, sp)
        b = run(geom, op, inp, ang, opt, sp)
        assert np.array_equal(a, b)


def test_cone_flat_full_geometry_subset_of_views(golden3d, oracle_mod):
    """256^3 volume, 512 x 384 detector, SID 500 / SDD 1000 (the cone-beam
    configuration), on 4 of its 360 views: GPU against the reference's
    outputs (subsampled) and the FP32 oracle."""
    opt, ang = cases3d.cone_256cube()
    sel = cases3d.CONE_VIEWS
    x = cases3d.ellipsoids(256, 256, 256, 12, 4)[None]
    assert float(x.sum(dtype=np.float64)) == float(golden3d["cone256/x_sum"])
    out = run("cone_flat", "proj", x, ang[sel], opt)
    e = rel_l2(out[cases3d.CONE_SINO_STRIDE], golden3d["cone256/proj/ref"])
    eo = rel_l2(out, oracle_mod.run3d("cone_flat", "proj", x, ang[sel], opt, prec="f", nthreads=8))
    print(f"cone-flat 256^3 proj, 4 views: rel-L2 vs reference CUDA {e:.2e}, vs FP32 oracle {eo:.2e}")
    assert e <= 1e-5 and eo <= 5e-5
    y = np.random.default_rng(5).random((1, sel.size, 384, 512)).astype(np.float32)
    bt = run("cone_flat", "proj_t", y, ang[sel], opt)
    e = rel_l2(bt[cases3d.CONE_VOL_STRIDE], golden3d["cone256/proj_t/ref"])
    eo = rel_l2(bt, oracle_mod.run3d("cone_flat", "proj_t", y, ang[sel], opt, prec="f", nthreads=8))
    print(f"cone-flat 256^3 proj_t, 4 views: rel-L2 vs reference CUDA {e:.2e}, vs FP32 oracle {eo:.2e}")
    assert e <= 1e-5 and eo <= 5e-5


def test_spiral_full_geometry_subset_of_views(golden3d, oracle_mod):
    """512 x 512 x 128 volume at 0.66 x 0.66 x 1.0 mm, 64 x 736 arc detector,
    1152 views per turn, pitch 1 (the spiral configuration), on 6 of its
    3456 views: GPU against the reference's outputs (subsampled) and the FP32
    oracle."""
    opt, ang, sp = cases3d.spiral_512x128()
    sel = cases3d.SPIRAL_VIEWS
    sps = sp[:, sel].copy()
    x = cases3d.ellipsoids(128, 512, 512, 12, 6, 0.04)[None]
    assert float(x.sum(dtype=np.float64)) == float(golden3d["spiral512/x_sum"])
    out = run("spiral", "proj", x, ang[sel], opt, sps)
    e = rel_l2(out[cases3d.SPIRAL_SINO_STRIDE], golden3d["spiral512/proj/ref"])
    eo = rel_l2(out, oracle_mod.run3d("spiral", "proj", x, ang[sel], opt, source_pos=sps, prec="f", nthreads=8))
    print(f"spiral 512x512x128 proj, 6 views: rel-L2 vs reference CUDA {e:.2e}, vs FP32 oracle {eo:.2e}")
    assert e <= 1e-5 and eo <= 5e-5
    y = np.random.default_rng(7).random((1, sel.size, 64, 736)).astype(np.float32)
    bt = run("spiral", "proj_t", y, ang[sel], opt, sps)
    e = rel_l2(bt[cases3d.SPIRAL_VOL_STRIDE], golden3d["spiral512/proj_t/ref"])
    eo = rel_l2(bt, oracle_mod.run3d("spiral", "proj_t", y, ang[sel], opt, source_pos=sps, prec="f", nthreads=8))
    print(f"spiral 512x512x128 proj_t, 6 views: rel-L2 vs reference CUDA {e:.2e}, vs FP32 oracle {eo:.2e}")
    assert e <= 1e-5 and eo <= 5e-5


def _fuzz3d(n=12, seed=77):
    """Seeded random small 3-D geometries: volume and detector sizes, voxel
    aspect, SID / SDD, shifts, detector cells of 0.8 to 2.5 voxels at the
    isocentre (narrower cells make the comparison with the FP32 oracle, whose
    trigonometry rounds differently from the device's, ill-conditioned),
    random view angles, for spirals a random pitch and source table."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        geom = ("cone_flat", "cone_arc", "spiral")[i % 3]
        W, H = (int(v) for v in rng.integers(8, 49, 2))
        D = int(rng.integers(4, 25))
        px, py, pz = (float(v) for v in rng.uniform(0.6, 1.5, 3))
        sid = float(rng.uniform(250.0, 600.0))
        sdd = sid * float(rng.uniform(1.5, 2.2))
        mag = sdd / sid
        cw = max(px, py) * float(rng.uniform(0.8, 2.5))          # column width at the isocentre
        rw = pz * float(rng.uniform(0.8, 2.5))
        C = int(min(300, np.hypot(W * px, H * py) * 1.2 / cw) + 2)
        R = int(min(32, D * pz * 1.3 / rw) + 2) if geom != "spiral" else int(rng.integers(4, 12))
        col = cw * mag if geom == "cone_flat" else cw / sid
        row = rw * mag
        V = int(rng.integers(2, 13))
        ang = rng.uniform(0, 2 * np.pi, V).astype(np.float32)
        sh = rng.uniform(-0.4, 0.4, 5) * np.array([px, py, pz, cw, rw])
        if geom != "cone_flat":
            sh[3] /= sid                                         # arc column shift is an angle
        if geom == "spiral":
            opt = np.array([W, H, D, C, R, px, py, pz, col, row, sid, sdd, sh[0], sh[1], sh[3], sh[4]], np.float32)
            pitch = float(rng.uniform(0.2, 1.5))
            sp = spiral_source(V, pitch, -pitch * (V - 1) / 2, float(rng.uniform(-1, 1)),
                               float(rng.uniform(-1e-3, 1e-3)), float(rng.uniform(-0.2, 0.2)))
        else:
            opt = np.array([W, H, D, C, R, px, py, pz, col, row, sid, sdd] + list(sh), np.float32)
            sp = None
        out.append((geom, opt, ang, sp))
    return out


FUZZ3 = _fuzz3d()


@pytest.mark.parametrize("case", range(len(FUZZ3)))
def test_random_3d_geometries_match_oracle_and_are_adjoint(oracle_mod, case):
    """All 6 operators of each seeded random 3-D geometry against the FP32
    oracle (5e-5, as for the fixed small cases), and the dot test of each
    operator pair."""
    geom, opt, ang, sp = FUZZ3[case]
    x, y = cases3d.inputs((geom, opt, ang, sp), batch=2, seed=900 + case)
    outs = {}
    for op in cases3d.OPS:
        inp = x if op in cases3d.IMAGE_IN else y
        out = run(geom, op, inp, ang, opt, sp)
        ref = oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="f", nthreads=8)
        e = rel_l2(out, ref) if np.any(ref) else float(np.abs(out).max())
        assert e <= 5e-5, (case, geom, opt.tolist(), op, e)
        outs[op] = out.astype(np.float64)
    for fwd, adj in (("proj", "proj_t"), ("bproj_t", "bproj"), ("bproj_tw", "bproj_w")):
        lhs, rhs = float((outs[fwd] * y).sum()), float((x * outs[adj]).sum())
        assert abs(lhs - rhs) <= 1e-6 * max(abs(lhs), 1e-30), (case, fwd, lhs, rhs)


def _dot_and_fd(label, fwd, adj, x, ang_all, ang_fd, nvox=64, seed=0):
    """Dot test of (fwd, adj) on all of `ang_all` (FP64 accumulation) and
    central finite differences of ||A x - b||^2 on `ang_fd` at `nvox` voxels
    that the views see (the loss is quadratic and a voxel changes only the
    cells its rays cross, so FD carries no truncation error)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    ax = fwd(x, ang_all)
    y = torch.rand(ax.shape, device="cuda", generator=g)
    aty = adj(y, ang_all)
    lhs = float((ax.double() * y.double()).sum())
    rhs = float((x.double() * aty.double()).sum())
    dot = abs(lhs - rhs) / abs(lhs)
    del ax, y, aty
    b = fwd(x, ang_fd) * 0.9
    base = x * 1.05
    r = fwd(base, ang_fd) - b
    grad = 2.0 * adj(r, ang_fd)
    flat = grad.view(-1)
    cand = torch.nonzero(flat.abs() > 1e-3 * float(flat.abs().max())).view(-1)
    pick = cand[torch.randperm(cand.numel(), device="cuda", generator=g)[:nvox]]
    h = 1e-2 * float(x.abs().max())
    fd, ag = [], []
    for k in pick.tolist():
        e = torch.zeros_like(base).view(-1)
        e[k] = h
        e = e.view_as(base)
        lp = ((fwd(base + e, ang_fd) - b).double() ** 2).sum()
        lm = ((fwd(base - e, ang_fd) - b).double() ** 2).sum()
        fd.append(float((lp - lm) / (2 * h)))
        ag.append(float(flat[k]))
    err = rel_l2(np.array(ag), np.array(fd))
    print(f"{label}: dot rel {dot:.2e} ({ang_all.numel()} views), FD vs A^T at {len(fd)} voxels {err:.2e}")
    assert dot <= 1e-6
    assert err <= 1e-3


def test_cone_beam_configuration_dot_and_fd():
    """2 x 256^3, 512 x 384 detector, SID 500 / SDD 1000: the dot test on all
    360 views, finite differences on 36 of them."""
    from pridediff_gb300 import radontorch as RT
    opt, ang_np = cases3d.cone_256cube()
    ot = torch.tensor(opt)
    x = torch.from_numpy(np.stack([cases3d.ellipsoids(256, 256, 256, 12, s) for s in (4, 5)])[:, None]).cuda()
    ang = torch.from_numpy(ang_np).cuda()
    _dot_and_fd("cone-flat 2 x 256^3", lambda v, a: RT.ProjConeFlatDis3d(v, ot, a),
                lambda w, a: RT.ProjTransConeFlatDis3d(w, ot, a), x, ang, ang[::10].contiguous(), seed=4)


def test_spiral_configuration_dot_and_fd():
    """2 x 512 x 512 x 128, 64 x 736 arc detector, pitch 1: the dot test on
    the 1152 views of the middle turn, finite differences on 24 of them."""
    from pridediff_gb300 import radontorch as RT
    opt, ang_np, sp_np = cases3d.spiral_512x128()
    ot = torch.tensor(opt)
    turn = slice(1152, 2304)
    ang = torch.from_numpy(ang_np[turn].copy()).cuda()
    sp = torch.from_numpy(sp_np[:, turn].copy()).cuda()
    sel = torch.arange(0, 1152, 48, device="cuda")
    sps = {ang.numel(): sp, sel.numel(): sp[:, sel].contiguous()}
    x = torch.from_numpy(np.stack([cases3d.ellipsoids(128, 512, 512, 12, s, 0.04) for s in (6, 7)])[:, None]).cuda()
    _dot_and_fd("spiral 2 x 512x512x128", lambda v, a: RT.ProjSpiralDis3d(v, ot, a, sps[a.numel()]),
                lambda w, a: RT.ProjTransSpiralDis3d(w, ot, a, sps[a.numel()]), x, ang, ang[sel].contiguous(),
                seed=6)


def test_projector3d_autograd_gradient_is_the_adjoint():
    import pridediff_gb300 as P
    proj = P.projector3d((32, 28, 20), (48, 24), 1.0, 1.0, 300.0, 600.0, scan_type="flat").cuda()
    ang = torch.arange(16, dtype=torch.float32, device="cuda") * (2 * np.pi / 16)
    x = torch.rand((2, 1, 20, 28, 32), device="cuda", requires_grad=True)
    y = proj.projection(x, ang)
    w = torch.randn_like(y)
    (y * w).sum().backward()
    assert torch.equal(x.grad, proj.projection_t(w, ang))
    # central finite differences of the quadratic loss ||Ax - b||^2 at a few voxels
    b = torch.rand_like(y)
    x0 = x.detach().clone()
    xr = x0.clone().requires_grad_(True)
    ((proj.projection(xr, ang) - b) ** 2).sum().backward()
    rng = np.random.default_rng(3)
    h = 0.05
    for _ in range(8):
        idx = tuple(int(rng.integers(0, s)) for s in x0.shape)
        xp, xm = x0.clone(), x0.clone()
        xp[idx] += h
        xm[idx] -= h
        with torch.no_grad():
            lp = ((proj.projection(xp, ang) - b).double() ** 2).sum()
            lm = ((proj.projection(xm, ang) - b).double() ** 2).sum()
        fd = float((lp - lm) / (2 * h))
        g = float(xr.grad[idx])
        assert abs(fd - g) <= 1e-3 * max(1.0, abs(g))


def test_projectorsp_autograd_and_arc_flip():
    import pridediff_gb300 as P
    proj = P.projectorsp((24, 24, 16), (40, 8), (1.2, 1.2, 1.0), (1.6, 1.0), 300.0, 600.0).cuda()
    V = 20
    ang = torch.arange(V, dtype=torch.float32, device="cuda") * (2 * np.pi / 10)
    sp = torch.from_numpy(cases3d.spiral_source(V, 0.8, -8.0)).cuda()
    x = torch.rand((1, 2, 16, 24, 24), device="cuda", requires_grad=True)
    y = proj.projection(x, ang, sp)
    w = torch.randn_like(y)
    (y * w).sum().backward()
    assert torch.equal(x.grad, proj.projection_t(w, ang, sp))


def test_dc_step_3d_matches_separate_operators():
    import ctypes
    from pridediff_gb300 import _native as N
    from pridediff_gb300 import radontorch as RT
    geom, opt, ang, sp = CASES["spiral_blocks"]
    lib = N.load()
    g = N.geom3d([float(v) for v in opt], spiral=True)
    V = len(ang)
    B = 2
    x, y = cases3d.inputs(CASES["spiral_blocks"], batch=B, seed=23)
    xt = torch.from_numpy(x).cuda()
    yt = torch.from_numpy(y).cuda() * 10.0
    at = torch.from_numpy(ang).cuda()
    spt = torch.from_numpy(sp).cuda()
    plan = RT.plan3d("spiral", g, at, spt)
    nbytes = int(lib.dd3d_dc_workspace_bytes(2, g, B, V))
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    resid = torch.empty_like(yt)
    eta = 1e-3
    xs = xt.clone()
    st = lib.dd3d_dc_step(2, g, plan.data_ptr(), xs.data_ptr(), yt.data_ptr(), resid.data_ptr(),
                          ctypes.c_float(eta), B, V, ws.data_ptr(), nbytes, torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    ot = torch.tensor(opt)
    ax = RT.ProjSpiralDis3d(xt[:, None], ot, at, spt)[:, 0]
    assert torch.equal(resid, ax - yt)
    expect = xt - eta * RT.ProjTransSpiralDis3d((ax - yt)[:, None], ot, at, spt)[:, 0]
    assert rel_l2(xs.cpu().numpy(), expect.cpu().numpy()) <= 1e-6


def test_3d_errors():
    from pridediff_gb300 import radontorch as RT
    opt = torch.tensor([8, 8, 4, 16, 4, 1, 1, 1, 1, 1, 100, 200, 0, 0, 0, 0, 0], dtype=torch.float32)
    ang = torch.zeros(4, device="cuda")
    with pytest.raises(RuntimeError):
        RT.ProjConeFlatDis3d(torch.zeros((1, 1, 4, 8, 8)), opt, ang)            # CPU tensor
    with pytest.raises(RuntimeError):
        RT.ProjConeFlatDis3d(torch.zeros((1, 1, 4, 8, 9), device="cuda"), opt, ang)   # size mismatch
    bad = opt.clone()
    bad[5] = -1.0
    with pytest.raises(RuntimeError):
        RT.ProjConeFlatDis3d(torch.zeros((1, 1, 4, 8, 8), device="cuda"), bad, ang)   # negative pixel

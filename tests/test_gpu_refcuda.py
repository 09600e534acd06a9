"""GPU parity against deeprecon's own CUDA kernels, run on the same GPU.

deeprecon has no CPU path for cone-flat, cone-arc and spiral
(RadonTorch.cpp:604, :641, :1055): its CUDA kernels are the reference.  They
are compiled unmodified into oracle/_ref/cuda/*.fatbin (where the reference
sources exist) and launched by oracle/refcuda.py with the reference host
functions' texture staging, grids and stream.  The reference accumulates its
transposes with float atomics, so its outputs vary with the order of the
atomics by FP32 rounding; the bar is rel-L2 <= 1e-5.  The CPU oracle, which
rounds its trigonometry correctly where the device code calls CUDA's
single-precision functions, is held to 5e-5 against the same outputs.

In 2-D deeprecon's CPU path is the parity target (the operators are
bit-exact with it, test_gpu_2d.py); its CUDA path restarts the FP32
accumulation of the pixel boundaries in every block of 256 detector bins
where the CPU path accumulates over the whole line, so the two differ by up
to 1e-3 (relative L2) on 512-pixel lines.  The 2-D tests here show that the
operators sit exactly as far from the reference's CUDA path as the
reference's CPU path does.

Each case is first scanned on the CPU (oracle.scan_hazards): views where one
of the reference kernels' walk starts could round to index -1 (an
out-of-bounds shared-memory or output access in the reference's own code)
are not given to the reference.  The tests skip where the fatbins are
absent; tests/golden/dd3d_golden.npz holds the reference's outputs on the
small cases for machines without them (test_gpu_3d.py).
"""
import numpy as np
import pytest
import torch

import cases3d
from conftest import rel_l2

pytestmark = pytest.mark.gpu

refcuda = pytest.importorskip("oracle.refcuda")
if not refcuda.available():
    pytest.skip("reference CUDA fatbins absent (oracle/_ref/cuda)", allow_module_level=True)

NAMES3 = {"proj": "Proj{}Dis3d", "proj_t": "ProjTrans{}Dis3d", "bproj": "BackProj{}Dis3d",
          "bproj_t": "BackProjTrans{}Dis3d", "bproj_w": "BackProjWeighted{}Dis3d",
          "bproj_tw": "BackProjTransWeighted{}Dis3d"}
NAMES2 = {k: v.replace("3d", "2d") for k, v in NAMES3.items()}
GEO = {"cone_flat": "ConeFlat", "cone_arc": "ConeArc", "spiral": "Spiral",
       "para": "Para", "flat": "FanFlat", "arc": "FanArc"}
OPS2 = {"para": ["proj", "proj_t", "bproj", "bproj_t"],
        "flat": cases3d.OPS, "arc": cases3d.OPS}


def ours(geom, op, x, ang, opt, sp=None):
    from pridediff_gb300 import radontorch
    names = NAMES2 if geom in OPS2 else NAMES3
    fn = getattr(radontorch, names[op].format(GEO[geom]))
    ot = torch.tensor(np.asarray(opt, np.float32))
    return fn(x, ot, ang, sp) if geom == "spiral" else fn(x, ot, ang)


def both(geom, op, x_np, ang_np, opt, sp_np=None):
    """(ours, reference) outputs of one operator on the same device inputs."""
    import oracle
    assert oracle.scan_hazards(geom, ang_np, opt, sp_np).sum() == 0
    x = torch.from_numpy(np.ascontiguousarray(x_np, np.float32)).cuda()
    ang = torch.from_numpy(np.ascontiguousarray(ang_np, np.float32)).cuda()
    sp = None if sp_np is None else torch.from_numpy(np.ascontiguousarray(sp_np, np.float32)).cuda()
    a = ours(geom, op, x, ang, opt, sp)
    b = refcuda.run(geom, op, x, ang, opt, sp)
    torch.cuda.synchronize()
    return a.cpu().numpy(), b.cpu().numpy()


CASES3 = cases3d.cases()


@pytest.mark.parametrize("name", sorted(CASES3))
@pytest.mark.parametrize("op", cases3d.OPS)
def test_3d_small_cases_match_reference_cuda(oracle_mod, name, op):
    geom, opt, ang, sp = CASES3[name]
    x, y = cases3d.inputs(CASES3[name], batch=2, seed=31)
    inp = x if op in cases3d.IMAGE_IN else y
    a, b = both(geom, op, inp[:, None], ang, opt, sp)
    e = rel_l2(a, b)
    e64 = rel_l2(a[:, 0], oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="d", nthreads=8))
    eo = rel_l2(oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="f", nthreads=1), b[:, 0])
    print(f"{name} {op}: rel-L2 vs reference CUDA {e:.2e} (FP32 oracle vs reference CUDA {eo:.2e}), "
          f"vs FP64 oracle {e64:.2e}")
    assert e <= 1e-5
    assert eo <= 5e-5


@pytest.mark.parametrize("case,geom,op", [(c, c.split("_")[0], op)
                                          for c in ["para_small", "flat_small", "arc_small", "flat_odd"]
                                          for op in OPS2[c.split("_")[0]]])
def test_2d_golden_cases_against_reference_cuda(golden, oracle_mod, case, geom, op):
    """The 2-D golden cases on the views the reference kernels can be run on
    (all but 1 of flat_small's 120 and 5 of arc_small's 120)."""
    opt = golden[f"{case}/options"]
    ang = golden[f"{case}/angles"]
    keep = oracle_mod.safe_views(geom, ang, opt)
    assert keep.size >= ang.size - 5
    x = golden[f"{case}/image"] if op in cases3d.IMAGE_IN else golden[f"{case}/sino"][:, keep]
    _check_2d_against_reference_cuda(oracle_mod, f"{case} ({keep.size} of {ang.size} views)", geom, op, x,
                                     ang[keep], opt)


def _check_2d_against_reference_cuda(oracle_mod, label, geom, op, x, ang, opt):
    a, b = both(geom, op, x[:, None], ang, opt)
    cpu = oracle_mod.run2d(geom, op, x, ang, opt, "f", 16)   # bit-exact with deeprecon's CPU path
    e, e_cpu, e_ours_cpu = rel_l2(a, b), rel_l2(cpu, b[:, 0]), rel_l2(a[:, 0], cpu)
    print(f"{label} {op}: rel-L2 vs reference CUDA {e:.2e}; reference CPU vs reference CUDA {e_cpu:.2e}; "
          f"vs reference CPU {e_ours_cpu:.2e}")
    assert e_ours_cpu <= 1e-5
    assert e <= 1.05 * e_cpu + 1e-5


C4_OPT, C4_ANG = cases3d.cone_256cube()


def test_cone_flat_256cube_360_views_match_reference_cuda():
    """The cone-beam configuration (256^3, 512 x 384 detector, SID 500 /
    SDD 1000) on every view the reference can be run on (356 of 360: on 4
    views an image edge and a column boundary tie to within rounding)."""
    import oracle
    keep = oracle.safe_views("cone_flat", C4_ANG, C4_OPT)
    assert keep.size >= 350
    ang = C4_ANG[keep]
    x = cases3d.ellipsoids(256, 256, 256, 12, 4)[None, None]
    a, b = both("cone_flat", "proj", x, ang, C4_OPT)
    e = rel_l2(a, b)
    print(f"cone-flat 256^3 proj, {ang.size} views: rel-L2 vs reference CUDA {e:.2e}")
    assert e <= 1e-5
    y = np.random.default_rng(5).random(a.shape).astype(np.float32)
    a, b = both("cone_flat", "proj_t", y, ang, C4_OPT)
    e = rel_l2(a, b)
    print(f"cone-flat 256^3 proj_t, {ang.size} views: rel-L2 vs reference CUDA {e:.2e}")
    assert e <= 1e-5


def test_spiral_512x512x128_one_turn_matches_reference_cuda():
    """The spiral configuration (512 x 512 x 128 at 0.66 x 0.66 x 1 mm,
    64 x 736 arc detector, pitch 1, 1152 views per turn) on the middle turn's
    views that the reference can be run on."""
    import oracle
    opt, ang, sp = cases3d.spiral_512x128()
    keep = oracle.safe_views("spiral", ang, opt, sp)
    keep = keep[(keep >= 1152) & (keep < 2304)]
    assert keep.size >= 1100
    x = cases3d.ellipsoids(128, 512, 512, 12, 6, 0.04)[None, None]
    a, b = both("spiral", "proj", x, ang[keep], opt, sp[:, keep])
    e = rel_l2(a, b)
    print(f"spiral 512x512x128 proj, {keep.size} views: rel-L2 vs reference CUDA {e:.2e}")
    assert e <= 1e-5
    y = np.random.default_rng(8).random(a.shape).astype(np.float32)
    a, b = both("spiral", "proj_t", y, ang[keep], opt, sp[:, keep])
    e = rel_l2(a, b)
    print(f"spiral 512x512x128 proj_t, {keep.size} views: rel-L2 vs reference CUDA {e:.2e}")
    assert e <= 1e-5


C2_OPT = np.array([512, 512, 736, 0.66, 0.66, 1.2858, 595.0, 1085.6, 0.0, 0.0, 0.0], np.float32)
C2_ANG = (np.arange(720) * 2 * np.pi / 720).astype(np.float32)


@pytest.mark.parametrize("op", cases3d.OPS)
def test_fan_flat_512_720_views_against_reference_cuda(oracle_mod, op):
    """The fan-beam batch configuration's geometry, 2 slices, all 6 operators."""
    rng = np.random.default_rng(12)
    if op in cases3d.IMAGE_IN:
        x = (rng.random((2, 512, 512)) * 0.04).astype(np.float32)
    else:
        x = rng.standard_normal((2, 720, 736)).astype(np.float32)
    _check_2d_against_reference_cuda(oracle_mod, "fan-flat 512^2 720 views", "flat", op, x, C2_ANG, C2_OPT)

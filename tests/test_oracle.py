"""The CPU oracle is pinned to deeprecon's own projectors.

* 2-D, against the golden vectors of deeprecon's CPU path (committed under
  tests/golden/, generated by tests/golden/make_golden.py): runs everywhere;
  bit-exact against the live reference build (oracle/_ref) where the
  reference sources were available at build time (skipped elsewhere).
* 3-D, against the outputs of deeprecon's CUDA kernels (the only 3-D
  implementation it has) in tests/golden/dd3d_golden.npz, made on a GB300 by
  make_golden.py --cuda3d: within 5e-5 relative L2 (the oracle rounds its
  trigonometry correctly; the reference's device code calls CUDA's
  single-precision sin, cos, tan and atan).
* The start-index scan that decides which views the reference kernels may be
  run on (oracle.scan_hazards).
"""
import numpy as np
import pytest

from conftest import rel_l2

CASES = ["para_small", "flat_small", "arc_small", "flat_odd"]
OPS = {"para": ["proj", "proj_t", "bproj", "bproj_t"],
       "flat": ["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"],
       "arc": ["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"]}


def _cases():
    for c in CASES:
        geom = c.split("_")[0]
        for op in OPS[geom]:
            yield c, geom, op


@pytest.mark.parametrize("case,geom,op", list(_cases()))
def test_oracle_fp32_matches_golden(golden, oracle_mod, case, geom, op):
    opt = golden[f"{case}/options"]
    ang = golden[f"{case}/angles"]
    x = golden[f"{case}/image"] if op in oracle_mod.IMAGE_INPUT else golden[f"{case}/sino"]
    ref = golden[f"{case}/{op}/ref"]
    out = oracle_mod.run2d(geom, op, x, ang, opt, "f", 1)
    # bit-exact on the machine that made the vectors; libm differences between
    # x86-64 and aarch64 may move a trigonometric value by one ulp elsewhere
    assert rel_l2(out, ref) <= 2e-6


@pytest.mark.parametrize("case,geom,op", list(_cases()))
def test_oracle_fp64_close_to_golden(golden, oracle_mod, case, geom, op):
    opt = golden[f"{case}/options"]
    ang = golden[f"{case}/angles"]
    x = golden[f"{case}/image"] if op in oracle_mod.IMAGE_INPUT else golden[f"{case}/sino"]
    ref = golden[f"{case}/{op}/ref"]
    out = oracle_mod.run2d(geom, op, x, ang, opt, "d", 1)
    # the reference's own FP32 error (drifting boundaries, FP32 angles in the
    # arc geometry) bounds this; it is a sanity bound, not the parity bar
    assert rel_l2(out, ref) <= (3e-4 if geom == "arc" else 5e-5)


@pytest.mark.parametrize("case,geom,op", list(_cases()))
def test_oracle_fp32_bit_exact_vs_live_reference(golden, oracle_mod, case, geom, op):
    if not oracle_mod.have_ref():
        pytest.skip("reference CPU build not present on this machine")
    opt = golden[f"{case}/options"]
    ang = golden[f"{case}/angles"]
    x = golden[f"{case}/image"] if op in oracle_mod.IMAGE_INPUT else golden[f"{case}/sino"]
    ref = oracle_mod.ref2d(geom, op, x, ang, opt)
    out = oracle_mod.run2d(geom, op, x, ang, opt, "f", 1)
    np.testing.assert_array_equal(out, ref)


def test_golden_vectors_are_the_reference(golden, oracle_mod):
    if not oracle_mod.have_ref():
        pytest.skip("reference CPU build not present on this machine")
    for case, geom, op in _cases():
        opt = golden[f"{case}/options"]
        ang = golden[f"{case}/angles"]
        x = golden[f"{case}/image"] if op in oracle_mod.IMAGE_INPUT else golden[f"{case}/sino"]
        np.testing.assert_array_equal(oracle_mod.ref2d(geom, op, x, ang, opt), golden[f"{case}/{op}/ref"])


def test_oracle_multithreaded_forward_is_deterministic(oracle_mod):
    rng = np.random.default_rng(3)
    opt = [96, 80, 120, 0.7, 0.7, 1.0, 500.0, 900.0, 0.0, 0.0, 0.0]
    ang = (np.arange(300) * 2 * np.pi / 300).astype(np.float32)
    img = rng.random((2, 80, 96)).astype(np.float32)
    a = oracle_mod.run2d("flat", "proj", img, ang, opt, "f", 1)
    b = oracle_mod.run2d("flat", "proj", img, ang, opt, "f", 3)
    np.testing.assert_array_equal(a, b)


def test_oracle_rejects_invalid(oracle_mod):
    with pytest.raises(ValueError):
        oracle_mod.run2d("para", "bproj_w", np.zeros((1, 4, 4), np.float32),
                         np.zeros(3, np.float32), [4, 4, 5, 1, 1, 1, 1, 2, 0, 0, 0])


import cases3d  # noqa: E402


@pytest.fixture(scope="module")
def golden3d():
    import os
    from conftest import ROOT
    return np.load(os.path.join(ROOT, "tests", "golden", "dd3d_golden.npz"))


@pytest.mark.parametrize("name", sorted(cases3d.cases()))
def test_oracle_3d_pinned_to_reference_cuda(golden3d, oracle_mod, name):
    geom, opt, ang, sp = cases3d.cases()[name]
    x, y = cases3d.inputs(cases3d.cases()[name], batch=1, seed=31)
    for op in cases3d.OPS:
        inp = x if op in cases3d.IMAGE_IN else y
        out = oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="f", nthreads=4)
        e = rel_l2(out, golden3d[f"{name}/{op}/ref"])
        print(f"{name} {op}: FP32 oracle vs reference CUDA {e:.2e}")
        assert e <= 5e-5


def test_oracle_3d_full_geometries_pinned_to_reference_cuda(golden3d, oracle_mod):
    opt, ang = cases3d.cone_256cube()
    sel = cases3d.CONE_VIEWS
    x = cases3d.ellipsoids(256, 256, 256, 12, 4)[None]
    assert float(x.sum(dtype=np.float64)) == float(golden3d["cone256/x_sum"])
    out = oracle_mod.run3d("cone_flat", "proj", x, ang[sel], opt, prec="f", nthreads=8)
    assert rel_l2(out[cases3d.CONE_SINO_STRIDE], golden3d["cone256/proj/ref"]) <= 5e-5
    opt, ang, sp = cases3d.spiral_512x128()
    sel = cases3d.SPIRAL_VIEWS
    x = cases3d.ellipsoids(128, 512, 512, 12, 6, 0.04)[None]
    assert float(x.sum(dtype=np.float64)) == float(golden3d["spiral512/x_sum"])
    out = oracle_mod.run3d("spiral", "proj", x, ang[sel], opt, source_pos=sp[:, sel].copy(), prec="f", nthreads=8)
    assert rel_l2(out[cases3d.SPIRAL_SINO_STRIDE], golden3d["spiral512/proj/ref"]) <= 5e-5


def test_scan_flags_the_near_ties_of_the_cone_beam_configuration(oracle_mod):
    """On the 256^3 cone-beam geometry four views put an image edge within a
    few ulps of the first column boundary of a detector block: those are the
    views the reference kernels are not run on."""
    opt, ang = cases3d.cone_256cube()
    per = oracle_mod.scan_hazards("cone_flat", ang, opt)
    assert list(np.flatnonzero(per)) == [12, 102, 168, 258]
    assert oracle_mod.scan_hazards("para", ang, [256, 256, 367, 1, 1, 1, 500, 1000, 0, 0, 0]).sum() == 0
    for name, (geom, o, a, sp) in cases3d.cases().items():
        assert oracle_mod.scan_hazards(geom, a, o, sp).sum() == 0, name


def test_scan_counts_a_start_that_rounds_below_zero(oracle_mod):
    """A fan-flat view whose image edge sits exactly on the first detector
    boundary: the flat start formula is evaluated on both sides of the tie."""
    # view 0: the first column boundary maps to x = -(D/2) * ds * R / SDD at
    # the isocentre; an image whose left edge is there ties at its middle line
    D, ds, R, SDD = 64, 1.0, 500.0, 1000.0
    edge = D / 2 * ds * R / SDD
    W = 40
    sx = 2 * edge / W
    opt = [W, 41, D, sx, 1.0, ds, R, SDD, 0.0, 0.0, 0.0]
    per = oracle_mod.scan_hazards("flat", np.zeros(1, np.float32), opt)
    assert per[0] >= 1


def test_bench_comparator_views_are_the_scan_safe_views(oracle_mod):
    """bench.py's plain-GPU comparator runs deeprecon's kernels on fixed view
    lists; they must be exactly the views the scan finds safe."""
    import bench
    cone, spiral = bench.comparator_views()
    opt, ang = cases3d.cone_256cube()
    assert np.array_equal(cone, oracle_mod.safe_views("cone_flat", ang, opt))
    opt, ang, sp = cases3d.spiral_512x128()
    safe = oracle_mod.safe_views("spiral", ang, opt, sp)
    assert np.array_equal(spiral, safe[(safe >= bench.SPIRAL_TURN[0]) & (safe < bench.SPIRAL_TURN[1])])
    assert oracle_mod.scan_hazards("flat", bench.angles_np(), bench.OPTIONS).sum() == 0

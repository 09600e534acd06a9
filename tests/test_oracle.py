"""The CPU oracle is pinned to deeprecon's own CPU projectors.

* Against the golden vectors (reference outputs committed under
  tests/golden/, generated by tests/golden/make_golden.py): runs everywhere.
* Against the live reference build (oracle/_ref): runs where the reference
  sources were available at build time (skipped elsewhere).
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

"""CPU checks of the GPU algorithm through its host model.

tests/native/dd_model2d.cpp compiles the kernels' own geometry header
(pridediff_gb300/csrc/dd_geom2d.cuh) on the host and evaluates the same
integral formulas the CUDA kernels use.  These tests pin, without a GPU:

* the drift-piece model of the reference's FP32 boundary recurrence;
* the bit-exact geometry replication and the integral formulas, against the
  reference's outputs (golden vectors), at the 1e-5 parity bar.
"""
import numpy as np
import pytest

from conftest import rel_l2

OPS = {"para": ["proj", "proj_t", "bproj", "bproj_t"],
       "flat": ["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"],
       "arc": ["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"]}


def _cases():
    for c in ["para_small", "flat_small", "arc_small", "flat_odd"]:
        geom = c.split("_")[0]
        for op in OPS[geom]:
            yield c, geom, op


@pytest.mark.parametrize("case,geom,op", list(_cases()))
def test_model_matches_reference(golden, host_model, case, geom, op):
    opt = golden[f"{case}/options"]
    ang = golden[f"{case}/angles"]
    x = golden[f"{case}/image"] if op in ("proj", "bproj_t", "bproj_tw") else golden[f"{case}/sino"]
    out = host_model.apply2d(geom, op, x, ang, opt)
    assert rel_l2(out, golden[f"{case}/{op}/ref"]) <= 1e-5


def test_piece_model_reproduces_fp32_recurrence(host_model):
    rng = np.random.default_rng(7)
    total_bad = 0
    for _ in range(3000):
        pint = float(np.float32(rng.uniform(0.05, 3.0)))
        v0 = float(np.float32(rng.uniform(-900.0, 50.0)))
        n = int(rng.integers(2, 1500))
        bad, npiece, flags, dev = host_model.check_pieces(v0, pint, 0, n)
        assert bad < 1000000, "locate() returned the wrong pixel"
        assert dev <= 1.0 + 1e-6          # only round-to-even tie entries differ, by one ulp
        total_bad += bad
        assert flags == 0 and npiece <= 32
    assert total_bad < 0.001 * 3000 * 750


def test_piece_model_edge_sequences(host_model):
    # sequences that cross zero, start exactly on powers of two, or are one long
    for v0, pint, n in [(-1.0, 0.5, 10), (0.0, 0.25, 9), (-4.0, 1.0, 9), (128.0, 0.66, 300),
                        (-256.0, 0.3, 2000), (-0.001, 0.001, 50), (5.0, 2.0, 1)]:
        bad, npiece, flags, dev = host_model.check_pieces(float(np.float32(v0)), float(np.float32(pint)), 0, n)
        assert bad < 1000000 and dev <= 1.0 + 1e-6


@pytest.mark.parametrize("case", ["para_sys", "flat_sys", "arc_sys"])
def test_model_sysmatrix_matches_reference(sysmat_golden, host_model, case):
    """The system-matrix line walk (dd_line2_sysmat) reproduces deeprecon's
    GetSysMatrix* builders entry for entry: same order, rows, columns and
    FP32 values."""
    geom = case.split("_")[0]
    rows, cols, vals = host_model.sysmatrix2d(geom, sysmat_golden[f"{case}/angles"], sysmat_golden[f"{case}/options"])
    assert np.array_equal(rows, sysmat_golden[f"{case}/rows"])
    assert np.array_equal(cols, sysmat_golden[f"{case}/cols"])
    assert np.array_equal(vals, sysmat_golden[f"{case}/vals"])

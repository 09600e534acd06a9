"""CPU checks of the 3-D GPU algorithm through its host model.

tests/native/dd_model3d.cpp compiles the 3-D kernels' geometry header
(pridediff_gb300/csrc/dd_geom3d.cuh) on the host and evaluates the
column-segment (forward-type) and pixel-segment (adjoint-type) walks the
CUDA kernels use.  The reference has no CPU path for 3-D, so the bar is the
3-D oracle (a restatement of deeprecon's CUDA kernels, parity unpinned
against them): rel-L2 <= 1e-6 in FP32 for all six operators and the three
geometries, including detectors wider than one 256-column walk block, views
on the 45-degree branch boundary and flipped detectors.
"""
import numpy as np
import pytest

import cases3d
from conftest import rel_l2

CASES = cases3d.cases()


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("op", cases3d.OPS)
def test_model_matches_oracle(host_model3, oracle_mod, name, op):
    geom, opt, ang, sp = CASES[name]
    x, y = cases3d.inputs(CASES[name], batch=1, seed=3)
    inp = x if op in cases3d.IMAGE_IN else y
    out = host_model3.apply3d(geom, op, inp, ang, opt, sp)
    ref = oracle_mod.run3d(geom, op, inp, ang, opt, source_pos=sp, prec="f", nthreads=4)
    assert rel_l2(out, ref) <= 1e-6


@pytest.mark.parametrize("name", ["cone_flat_small", "spiral_small"])
def test_model_pairs_are_exact_transposes(host_model3, name):
    geom, opt, ang, sp = CASES[name]
    x, y = cases3d.inputs(CASES[name], batch=1, seed=5)
    for fwd, adj in (("proj", "proj_t"), ("bproj_t", "bproj"), ("bproj_tw", "bproj_w")):
        ax = host_model3.apply3d(geom, fwd, x, ang, opt, sp).astype(np.float64)
        aty = host_model3.apply3d(geom, adj, y, ang, opt, sp).astype(np.float64)
        lhs, rhs = float((ax * y).sum()), float((x * aty).sum())
        assert abs(lhs - rhs) <= 1e-6 * abs(lhs)

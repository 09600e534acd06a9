"""Edge sizes of the 2-D operators against the FP32 oracle: a single pixel, a
single view, the largest detector (1984 bins, the widest pass class), lines
of 4096 pixels (the forward then stages 1 image per CTA instead of 4),
batches that are not a multiple of the 4 images a CTA takes."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

# (geometry, W, H, D, V, B, pixel size, detector size, operators); fan images
# stay inside the source circle (SID 595 mm) and bins span a few pixels (the
# reference's sequential FP32 sum over a bin of hundreds of pixels is itself
# about 1e-5 from exact)
CASES = [
    ("flat", 1, 1, 3, 4, 1, 0.7, 1.3, ("proj", "proj_t")),
    ("flat", 5, 300, 7, 1, 3, 0.7, 1.3, ("proj", "proj_t", "bproj_tw")),
    ("arc", 130, 70, 1984, 8, 5, 0.7, 0.06 / 1085.6, ("proj", "proj_t", "bproj", "bproj_t")),
    ("flat", 4096, 3, 400, 6, 3, 0.1, 1.3, ("proj", "proj_t", "bproj_t", "bproj_tw")),
    ("para", 3, 4096, 50, 5, 2, 0.7, 1.0, ("proj", "proj_t")),
    ("flat", 64, 64, 90, 7, 9, 0.7, 1.3, ("proj", "proj_t", "bproj_w")),
]
NAMES = {"para": "Para", "flat": "FanFlat", "arc": "FanArc"}
OPS = {"proj": "Proj{}Dis2d", "proj_t": "ProjTrans{}Dis2d", "bproj": "BackProj{}Dis2d",
       "bproj_t": "BackProjTrans{}Dis2d", "bproj_w": "BackProjWeighted{}Dis2d",
       "bproj_tw": "BackProjTransWeighted{}Dis2d"}


@pytest.mark.parametrize("case", range(len(CASES)))
def test_edge_sizes_match_oracle(oracle_mod, case):
    from pridediff_gb300 import radontorch
    geom, W, H, D, V, B, pix, det, ops = CASES[case]
    opt = [W, H, D, pix, 0.85 * pix, det, 595.0, 1085.6, 0.1, -0.2, 0.0]
    ang = (np.arange(V) * 2 * np.pi / max(V, 1) + 0.1).astype(np.float32)
    rng = np.random.default_rng(100 + case)
    for op in ops:
        x = rng.random((B, H, W), dtype=np.float32) if op in oracle_mod.IMAGE_INPUT else \
            rng.standard_normal((B, V, D)).astype(np.float32)
        ref = oracle_mod.run2d(geom, op, x, ang, opt)
        fn = getattr(radontorch, OPS[op].format(NAMES[geom]))
        out = fn(torch.from_numpy(x)[:, None].cuda(), torch.tensor(opt), torch.from_numpy(ang).cuda())
        got = out[:, 0].cpu().numpy()
        assert got.shape == ref.shape, (op, got.shape, ref.shape)
        err = rel_l2(got, ref) if np.any(ref) else float(np.abs(got).max())
        assert err <= 1e-5, (geom, W, H, D, V, B, op, err)


def _fuzz_cases(n=30, seed=2026):
    """Seeded random geometries: sizes, pixel aspect, shifts, detector cells of
    0.5 to 3 pixels, views at random angles plus exact multiples of 45 degrees."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        geom = ("para", "flat", "arc")[i % 3]
        W, H = (int(v) for v in rng.integers(8, 301, 2))
        pix = float(rng.uniform(0.4, 1.5))
        piy = pix * float(rng.uniform(0.7, 1.3))
        V = int(rng.integers(1, 41))
        B = int(rng.integers(1, 7))
        cell = pix * float(rng.uniform(0.5, 3.0))      # cell width at the isocentre
        extent = np.hypot(W * pix, H * piy) * (1.2 if geom == "para" else 2.0)
        D = int(min(max(8, extent / cell), 1984))
        det = cell if geom == "para" else (cell * 1085.6 / 595.0 if geom == "flat" else cell / 595.0)
        shifts = [float(v) for v in rng.uniform(-0.5, 0.5, 3) * np.array([pix, piy, cell])]
        if geom == "arc":
            shifts[2] /= 595.0          # the arc detector's shift is an angle, like its cells
        ang = rng.uniform(0, 2 * np.pi, V)
        ang[: min(V, 4)] = np.arange(min(V, 4)) * np.pi / 4   # 0, 45, 90, 135 degrees
        opt = [W, H, D, pix, piy, det, 595.0, 1085.6] + shifts
        out.append((geom, opt, ang.astype(np.float32), B))
    return out


FUZZ = _fuzz_cases()


@pytest.mark.parametrize("case", range(len(FUZZ)))
def test_random_geometries_match_oracle(oracle_mod, case):
    """Every operator of each seeded random 2-D geometry against the FP32
    oracle (bit-exact with deeprecon's CPU code) at 1e-5."""
    from pridediff_gb300 import radontorch
    geom, opt, ang, B = FUZZ[case]
    W, H, D = (int(v) for v in opt[:3])
    V = ang.size
    ops = ["proj", "proj_t", "bproj", "bproj_t"] + ([] if geom == "para" else ["bproj_w", "bproj_tw"])
    rng = np.random.default_rng(500 + case)
    for op in ops:
        x = rng.random((B, H, W), dtype=np.float32) if op in oracle_mod.IMAGE_INPUT else \
            rng.standard_normal((B, V, D)).astype(np.float32)
        ref = oracle_mod.run2d(geom, op, x, ang, np.asarray(opt, np.float32))
        fn = getattr(radontorch, OPS[op].format(NAMES[geom]))
        got = fn(torch.from_numpy(x)[:, None].cuda(), torch.tensor(opt, dtype=torch.float32),
                 torch.from_numpy(ang).cuda())[:, 0].cpu().numpy()
        assert got.shape == ref.shape, (op, got.shape, ref.shape)
        err = rel_l2(got, ref) if np.any(ref) else float(np.abs(got).max())
        assert err <= 1e-5, (case, geom, opt, V, B, op, err)

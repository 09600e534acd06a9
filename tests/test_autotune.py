"""The autotuner's persistence (CPU only: measurements are injected)."""
import json
import multiprocessing as mp
import os

import pytest

from pridediff_gb300 import autotune


def _fake_measure(cfg):
    return 1.0 + abs(cfg["ctas_per_sm"] - 2) + 0.5 * (1 - cfg["lpt_order"]) + 0.25 * (cfg["items_cluster"] - 1)


def test_tune_picks_fastest_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    calls = []

    def meas(cfg):
        calls.append(cfg)
        return _fake_measure(cfg)

    best = autotune.tune("k", autotune.BATCH_CANDIDATES, meas, path=path)
    assert best == {"ctas_per_sm": 2, "lpt_order": 1, "items_cluster": 1}
    assert len(calls) == len(autotune.BATCH_CANDIDATES)
    calls.clear()
    assert autotune.tune("k", autotune.BATCH_CANDIDATES, meas, path=path) == best
    assert calls == []   # served from the cache


def _worker_killed_mid_trial(path, stop_after):
    n = {"k": 0}

    def meas(cfg):
        n["k"] += 1
        if n["k"] > stop_after:
            os._exit(3)   # the process dies in the middle of a trial
        return _fake_measure(cfg)

    autotune.tune("resume", autotune.BATCH_CANDIDATES, meas, path=path)


def test_tuning_resumes_after_a_killed_worker(tmp_path):
    path = str(tmp_path / "tune.json")
    ctx = mp.get_context("spawn")
    p = ctx.Process(target=_worker_killed_mid_trial, args=(path, 3))
    p.start()
    p.join(60)
    assert p.exitcode == 3
    done = autotune.recorded("resume", path=path)
    assert len(done) == 3                      # the finished trials survived
    calls = []

    def meas(cfg):
        calls.append(cfg)
        return _fake_measure(cfg)

    best = autotune.tune("resume", autotune.BATCH_CANDIDATES, meas, path=path)
    assert len(calls) == len(autotune.BATCH_CANDIDATES) - 3   # only the missing ones
    assert best == {"ctas_per_sm": 2, "lpt_order": 1, "items_cluster": 1}


def test_corrupt_cache_is_discarded(tmp_path):
    path = str(tmp_path / "tune.json")
    with open(path, "w") as f:
        f.write('{"format": 1, "entries": {"x": ')      # truncated write
    best = autotune.tune("k", autotune.BATCH_CANDIDATES, _fake_measure, path=path)
    assert best["ctas_per_sm"] == 2
    with open(path) as f:
        assert json.load(f)["format"] == 1


def test_keys_separate_problems(tmp_path):
    a = autotune.make_key(kind="x", shapes=[(1, 2)], gpu="G")
    b = autotune.make_key(kind="x", shapes=[(1, 3)], gpu="G")
    assert a != b and a == autotune.make_key(gpu="G", shapes=[(1, 2)], kind="x")


@pytest.mark.gpu
def test_gpu_every_forward_shape_is_the_same_operator(oracle_mod, tmp_path, monkeypatch):
    """The single-geometry forward's tunable CTA shapes (4 or 1 slices per
    CTA, a view's lines on a cluster of 2 CTAs or on 1) compute the same
    projection: the slice grouping does not touch the arithmetic (bit-equal),
    the cluster changes the order of one sum (FP32 rounding); each matches the
    reference CPU path.  The first forward of a geometry runs the tuner and
    records its choice."""
    import numpy as np
    import torch
    from conftest import rel_l2
    from pridediff_gb300 import _native as N
    from pridediff_gb300 import radontorch as RT
    monkeypatch.setenv("PRIDEDIFF_TUNE_CACHE", str(tmp_path / "tune.json"))
    lib = N.load()
    opt = [96, 80, 130, 0.9, 0.9, 1.3, 595.0, 1085.6, 0.2, -0.1, 0.3]
    g = N.geom2d(opt)
    V, B = 90, 5
    ang_np = (np.arange(V) * 2 * np.pi / V).astype(np.float32)
    x_np = np.random.default_rng(2).random((B, 80, 96)).astype(np.float32)
    x, ang = torch.from_numpy(x_np).cuda(), torch.from_numpy(ang_np).cuda()
    plan = RT.plan2d("flat", g, ang)
    nbytes = int(lib.dd2d_apply_workspace_bytes(1, 0, g, B, V))
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    ref = oracle_mod.run2d("flat", "proj", x_np, ang_np, opt, "f", 0)
    outs = {}
    for cfg in autotune.FORWARD2D_CANDIDATES:
        out = torch.empty((B, V, 130), device="cuda")
        st = lib.dd2d_apply_planned_tuned(1, 0, g, plan.data_ptr(), x.data_ptr(), out.data_ptr(), B, V,
                                          ws.data_ptr(), nbytes, RT.forward_tune(cfg),
                                          torch.cuda.current_stream().cuda_stream)
        assert st == 0
        torch.cuda.synchronize()
        outs[(cfg["fwd_slices"], cfg["fwd_cluster"])] = out
        assert rel_l2(out.cpu().numpy(), ref) <= 1e-5
    for cl in (1, 2):
        assert torch.equal(outs[(4, cl)], outs[(1, cl)])
    assert rel_l2(outs[(4, 1)].cpu().numpy(), outs[(4, 2)].cpu().numpy()) <= 1e-6
    y = RT.ProjFanFlatDis2d(x[:, None], torch.tensor(opt), ang)
    rec = [r for r in autotune.chosen() if r.get("image") == [96, 80] and r.get("batch") == B]
    assert rec and rec[0]["choice"] in autotune.FORWARD2D_CANDIDATES
    assert len(rec[0]["trials"]) == len(autotune.FORWARD2D_CANDIDATES)
    assert torch.equal(y[:, 0], outs[(rec[0]["choice"]["fwd_slices"], rec[0]["choice"]["fwd_cluster"])])

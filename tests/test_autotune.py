"""The autotuner's persistence (CPU only: measurements are injected)."""
import json
import multiprocessing as mp
import os

import pytest

from pridediff_gb300 import autotune


def _fake_measure(cfg):
    return 1.0 + abs(cfg["ctas_per_sm"] - 2) + 0.5 * (1 - cfg["lpt_order"])


def test_tune_picks_fastest_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    calls = []

    def meas(cfg):
        calls.append(cfg)
        return _fake_measure(cfg)

    best = autotune.tune("k", autotune.BATCH_CANDIDATES, meas, path=path)
    assert best == {"ctas_per_sm": 2, "lpt_order": 1}
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
    assert best == {"ctas_per_sm": 2, "lpt_order": 1}


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

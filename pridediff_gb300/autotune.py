"""Project autotuner for the launch shapes of the kernels.

Two problems are tuned: the single-geometry forward's CTA shape (slices per
CTA and the size of the cluster that shares a view's walked lines --
``tune_forward2d``, run by the radontorch operators on the first forward of a
geometry and batch) and the persistent uneven batch's launch (CTAs per SM,
item order, cluster size per item -- ``tune_batch_dc``).

A tuning problem is a key (what is being run: scan type, instance shapes,
GPU, driver, library version) and a list of candidate configurations; the
measure function returns seconds per call of one candidate.  Every finished
trial is written to a JSON cache immediately (atomic replace), so a tuning
run that is interrupted -- the process killed mid-trial -- resumes from the
trials already recorded, and a corrupt or truncated cache file is discarded
rather than trusted.  Once every candidate of a key has a time, the best one
is stored as the key's choice and returned without measuring again.

Cache location: $PRIDEDIFF_TUNE_CACHE, else ~/.cache/pridediff_gb300/tune.json.
"""
from __future__ import annotations

import hashlib
import json
import os
import tempfile
import threading
from typing import Callable, Dict, List, Optional

_lock = threading.Lock()


def cache_path() -> str:
    p = os.environ.get("PRIDEDIFF_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "pridediff_gb300", "tune.json")


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        if not isinstance(data, dict) or data.get("format") != 1 or not isinstance(data.get("entries"), dict):
            return {"format": 1, "entries": {}}
        return data
    except (OSError, ValueError):
        return {"format": 1, "entries": {}}


def _store(path: str, data: dict) -> None:
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d or ".", prefix=".tune.", suffix=".tmp")
    try:
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.flush()
            os.fsync(f.fileno())
        os.replace(tmp, path)
    finally:
        if os.path.exists(tmp):
            os.unlink(tmp)


def make_key(**parts) -> str:
    blob = json.dumps(parts, sort_keys=True, default=str)
    return hashlib.sha1(blob.encode()).hexdigest()[:20]


def _cfg_id(cfg: dict) -> str:
    return json.dumps(cfg, sort_keys=True)


def tune(key: str, candidates: List[dict], measure: Callable[[dict], float],
         path: Optional[str] = None, describe: Optional[dict] = None) -> dict:
    """Best candidate for `key`, measuring only candidates without a recorded time."""
    path = path or cache_path()
    with _lock:
        data = _load(path)
        ent = data["entries"].setdefault(key, {"trials": {}, "best": None, "about": describe or {}})
        if ent.get("best") is not None and all(_cfg_id(c) in ent["trials"] for c in candidates):
            return json.loads(ent["best"])
    for cfg in candidates:
        cid = _cfg_id(cfg)
        with _lock:
            data = _load(path)
            ent = data["entries"].setdefault(key, {"trials": {}, "best": None, "about": describe or {}})
            if cid in ent["trials"]:
                continue
        t = float(measure(cfg))
        with _lock:
            data = _load(path)
            ent = data["entries"].setdefault(key, {"trials": {}, "best": None, "about": describe or {}})
            ent["trials"][cid] = t
            _store(path, data)
    with _lock:
        data = _load(path)
        ent = data["entries"][key]
        best = min(((t, c) for c, t in ent["trials"].items() if c in {_cfg_id(x) for x in candidates}),
                   key=lambda p: p[0])
        ent["best"] = best[1]
        _store(path, data)
        return json.loads(best[1])


def recorded(key: str, path: Optional[str] = None) -> Dict[str, float]:
    return dict(_load(path or cache_path())["entries"].get(key, {}).get("trials", {}))


# ---------------------------------------------------------------------------
# GPU problems
# ---------------------------------------------------------------------------
# ctas_per_sm 0: as many persistent CTAs as fit on an SM
BATCH_CANDIDATES = [{"ctas_per_sm": c, "lpt_order": o, "items_cluster": k}
                    for c in (0, 2, 4) for o in (1, 0) for k in (1, 2)]
# single-geometry forward: slices per CTA x CTAs per view's cluster
FORWARD2D_CANDIDATES = [{"fwd_slices": b, "fwd_cluster": c} for b in (4, 1) for c in (2, 1)]


def enabled() -> bool:
    """Autotuning of the single-geometry forward on first use (PRIDEDIFF_AUTOTUNE=0 turns it off)."""
    return os.environ.get("PRIDEDIFF_AUTOTUNE", "1") != "0"


def gpu_signature(device) -> dict:
    import torch
    from . import _native
    p = torch.cuda.get_device_properties(device)
    return {"gpu": p.name, "sm": f"{p.major}.{p.minor}", "sms": p.multi_processor_count,
            "cuda": torch.version.cuda, "lib": _native.load().dd_version().decode()}


def tune_batch_dc(batch, x, y, eta: float = 0.0, reps: int = 3, candidates=None, path=None) -> dict:
    """Pick the persistent-launch shape of an UnevenBatch2d's DC step."""
    import torch
    candidates = candidates or BATCH_CANDIDATES
    shapes = [(int(i.geom.width), int(i.geom.height), int(i.geom.num_det), int(i.num_view), int(i.batch))
              for i in batch.inst]
    key = make_key(kind="batch2d_dc", scan=batch.scan, shapes=shapes, **gpu_signature(batch.device))

    def measure(cfg):
        batch.set_tune(cfg)
        xs = x.clone()
        batch.dc_step(xs, y, eta)   # warm-up
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            batch.dc_step(xs, y, eta)
        b.record()
        torch.cuda.synchronize(batch.device)
        return a.elapsed_time(b) / 1e3 / reps

    best = tune(key, candidates, measure, path=path,
                describe={"kind": "batch2d_dc", "scan": batch.scan, "instances": len(shapes)})
    batch.set_tune(best)
    return best


_forward_choice: Dict[str, dict] = {}   # in-process copy of the cache's choices
_forward_about: Dict[str, dict] = {}    # what each key is


def forward2d_key(scan: int, geom_fields: tuple, batch: int, views: int, device) -> str:
    return make_key(kind="forward2d", scan=scan, geom=list(geom_fields), batch=batch, views=views,
                    **gpu_signature(device))


def tune_forward2d(key: str, run, reps: int = 3, path=None, about: Optional[dict] = None) -> dict:
    """Pick the single-geometry forward's CTA shape for one (geometry, batch):
    `run(cfg)` enqueues one forward with that shape on the current stream."""
    import torch
    if key in _forward_choice:
        return _forward_choice[key]
    _forward_about[key] = about or {}

    def measure(cfg):
        run(cfg)   # warm-up (kernel attributes)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            run(cfg)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / reps

    best = tune(key, FORWARD2D_CANDIDATES, measure, path=path, describe={"kind": "forward2d", **(about or {})})
    _forward_choice[key] = best
    return best


def chosen() -> List[dict]:
    """The forward shapes chosen in this process: what was tuned, the shape
    picked and the time of every candidate (seconds per call)."""
    return [{**_forward_about.get(k, {}), "choice": v, "trials": recorded(k)} for k, v in _forward_choice.items()]

#!/usr/bin/env python
"""Benchmark: batched fan-beam DD forward + matched-adjoint backward with autograd.

Workload (the reference's headline configuration for this path): 16 FP32
512x512 slices, pixel 0.66 mm, 720 views over 360 deg, 736 detector cells of
1.2858 mm, source-isocentre 595 mm, source-detector 1085.6 mm (fan-flat);
seeded random-ellipse phantoms scaled to mu in [0, 0.04] /mm; loss
||Ax - y||^2 with y = -log(max(Poisson(1e5 exp(-A x_true)), 1) / 1e5).  One
step = loss + loss.backward(): one forward projection A x and one exact
adjoint A^T r for every slice, through projector2d and its autograd pair.

Metric: FP+BP per second (slice forward + adjoint pairs per second).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times deeprecon's CPU algorithm on this host (the oracle
port of it; the reference sources are not present here) on the same
workload, a bounded sample of slices per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "FP+BP/s and %HBM roofline, batched+autograd vs plain GPU, rel err ≤1e-5"
UNIT = "FP+BP/s"
GEOM = dict(image=512, num_det=736, pix=0.66, det=1.2858, sid=595.0, sdd=1085.6, views=720, batch=16)
OPTIONS = [512, 512, 736, 0.66, 0.66, 1.2858, 595.0, 1085.6, 0.0, 0.0, 0.0]


def phantom(h, w, n, rng, scale):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.zeros((h, w))
    for _ in range(n):
        x0 = rng.uniform(-0.8, 0.8) * w / 2 + (w - 1) / 2
        y0 = rng.uniform(-0.8, 0.8) * h / 2 + (h - 1) / 2
        a, b = rng.uniform(5, 60), rng.uniform(5, 60)
        t = rng.uniform(0, np.pi)
        u = (xx - x0) * np.cos(t) + (yy - y0) * np.sin(t)
        v = -(xx - x0) * np.sin(t) + (yy - y0) * np.cos(t)
        img[(u / a) ** 2 + (v / b) ** 2 <= 1] += rng.uniform(0, 1)
    return np.clip(img * scale, 0, scale).astype(np.float32)


def angles_np():
    return (np.arange(GEOM["views"]) * 2 * np.pi / GEOM["views"]).astype(np.float32)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 9:
                continue
            for name, val in zip(names, r[5:9]):
                if val.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def cpu_port_baseline(seconds=10.0):
    """deeprecon's CPU algorithm (FP32 oracle port, reference thread rule) on one slice at a time."""
    import oracle
    oracle.build()
    rng = np.random.default_rng(99)
    ang = angles_np()
    img = phantom(512, 512, 10, rng, 0.04)[None]
    r = rng.standard_normal((1, GEOM["views"], GEOM["num_det"])).astype(np.float32)
    threads = oracle.default_threads(GEOM["views"])
    n = 0
    t0 = time.perf_counter()
    while True:
        oracle.run2d("flat", "proj", img, ang, OPTIONS, "f", threads)
        oracle.run2d("flat", "proj_t", r, ang, OPTIONS, "f", threads)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} slice(s) of the workload, forward + exact adjoint, {dt:.1f} s"}


def run_reference(args):
    """--impl reference: the CPU implementation on this host, same workload and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    rng = np.random.default_rng(99)
    ang = angles_np()
    threads = oracle.default_threads(GEOM["views"])
    per_step = 1   # slices per step (bounded sample: one slice of the 16-slice batch)
    imgs = [phantom(512, 512, 10, rng, 0.04)[None] for _ in range(per_step)]
    r = rng.standard_normal((1, GEOM["views"], GEOM["num_det"])).astype(np.float32)

    def step():
        for im in imgs:
            oracle.run2d("flat", "proj", im, ang, OPTIONS, "f", threads)
            oracle.run2d("flat", "proj_t", r, ang, OPTIONS, "f", threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = per_step * args.steps / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{per_step} slice per step (forward + exact adjoint), CPU"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def workload_config():
    return {"workload": "fan-flat DD FP + exact-adjoint BP with autograd, 16 x 512^2 slices, "
                        "720 views over 360 deg, 736 dets x 1.2858 mm, SID 595, SDD 1085.6",
            "global_batch": GEOM["batch"], "image": [512, 512], "views": 720, "num_det": 736,
            "scan_type": "flat", "l2": "flushed (256 MiB write) between timed steps",
            "parallelism": "replicas (instances sharded, no collective)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import pridediff_gb300 as P
    lib = P._native.load()

    B, V = GEOM["batch"], GEOM["views"]
    rng = np.random.default_rng(1234 + rank)
    proj = P.projector2d(512, 736, 0.66, 1.2858, 595.0, 1085.6, scan_type="flat").to(dev)
    ang = torch.from_numpy(angles_np()).to(dev)
    x_true = torch.from_numpy(np.stack([phantom(512, 512, 10, rng, 0.04) for _ in range(B)])[:, None]).to(dev)
    with torch.no_grad():
        p = proj.projection(x_true, ang)
        gen = torch.Generator(device=dev).manual_seed(4321 + rank)
        counts = torch.poisson(1e5 * torch.exp(-p.double()), generator=gen)
        y = (-torch.log(torch.clamp(counts, min=1.0) / 1e5)).float()
    x0 = (x_true * 0.8).contiguous()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step(x_in, y_in):
        x = x_in.detach().requires_grad_(True)
        loss = ((proj.projection(x, ang) - y_in) ** 2).sum()
        loss.backward()
        return x.grad, loss

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(max(args.warmup, 3)):
        step(x0, y)
    torch.cuda.synchronize()

    # ---- device-resident timing: per-step events, L2 flushed between steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    n0 = lib.dd_launch_count()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.fill_(float(i))
            starts[i].record()
            step(x0, y)
            stops[i].record()
        torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = (lib.dd_launch_count() - n0) // max(args.steps, 1)
    barrier()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, stops)) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * B / (ms / 1e3)

    # ---- dominant kernel: live CUDA-event timing of each launch
    lib.dd_profile_enable(1)
    for i in range(max(3, min(args.steps, 10))):
        flush.fill_(float(i))
        step(x0, y)
    torch.cuda.synchronize()
    kern = {}
    for kind, name in ((0, "k_fwd"), (1, "k_adj"), (2, "tables"), (3, "plan")):
        tot, cnt = P._native.ctypes.c_double(), P._native.ctypes.c_int()
        lib.dd_profile_read(kind, P._native.ctypes.byref(tot), P._native.ctypes.byref(cnt))
        if cnt.value:
            kern[name] = {"ms_per_launch": tot.value / cnt.value, "launches": cnt.value}
    lib.dd_profile_enable(0)
    peak, peak_kind = measured_peak_hbm()
    alg_bytes = 4.0 * V * (512 * 512 + 736) * B          # view-swept bytes per launch (B slices)
    dom = max(("k_fwd", "k_adj"), key=lambda k: kern.get(k, {}).get("ms_per_launch", 0.0))
    dom_ms = kern.get(dom, {}).get("ms_per_launch", float("nan"))
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9
    traffic = ncu_traffic().get(dom)

    # ---- end to end through the public API with host buffers
    x_host = x0.detach().cpu().pin_memory()
    y_host = y.detach().cpu().pin_memory()
    g_host = torch.empty_like(x_host).pin_memory()
    x_dev = torch.empty_like(x0)
    y_dev = torch.empty_like(y)
    e_s = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    e_e = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.fill_(float(i))
        e_s[i].record()
        x_dev.copy_(x_host, non_blocking=True)
        y_dev.copy_(y_host, non_blocking=True)
        g, _ = step(x_dev, y_dev)
        g_host.copy_(g, non_blocking=True)
        e_e[i].record()
    torch.cuda.synchronize()
    e2e_ms = sum(a.elapsed_time(b) for a, b in zip(e_s, e_e)) / args.steps
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = world * B / (e2e_ms / 1e3)

    if rank == 0:
        cpu = None if args.no_cpu_baseline else cpu_port_baseline()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s",
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "bytes_model": "view-swept 4*V*(H*W + D) per slice per operator"},
            "kernels": kern,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(x_host.numel() * 4 + y_host.numel() * 4),
                    "d2h_bytes_per_step": int(g_host.numel() * 4)},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "wall_s_timed_region": wall,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

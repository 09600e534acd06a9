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

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--no-extras]

On one GPU the line also carries `extra`: the same slices through the plain
per-slice path (the unbatched comparator), the parallel-beam configuration
(one 256^2 slice, 180 views, 367 detectors), the FBP of the 16 sinograms (fused
weight + filter kernel, then the weighted back-projection, beside the
reference's torch-convolution composition), the 24-instance uneven batched
data-consistency loop captured in a CUDA graph, and the 3-D cone-flat and
spiral configurations, each with its view-swept bytes against the measured
HBM peak.

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


def _ellipsoids(shape, n, seed, scale, dev):
    """Sum of n seeded random ellipsoids (intensity U[0, 1]) on the device."""
    import torch
    g = np.random.default_rng(seed)
    D, H, W = shape
    z = torch.arange(D, device=dev, dtype=torch.float32)[:, None, None]
    y = torch.arange(H, device=dev, dtype=torch.float32)[None, :, None]
    x = torch.arange(W, device=dev, dtype=torch.float32)[None, None, :]
    vol = torch.zeros(shape, device=dev)
    for _ in range(n):
        c = [g.uniform(0.2, 0.8) * s for s in (D, H, W)]
        a = [g.uniform(0.05, 0.3) * s for s in (D, H, W)]
        inside = ((z - c[0]) / a[0]) ** 2 + ((y - c[1]) / a[1]) ** 2 + ((x - c[2]) / a[2]) ** 2 <= 1
        vol += inside.float() * float(g.uniform(0, 1))
    return vol * scale


def _timed(fn, reps, flush, ev):
    """Mean ms of fn over reps, CUDA events on the current stream, L2 flushed before each."""
    import torch
    fn()
    torch.cuda.synchronize()
    tot = 0.0
    for i in range(reps):
        flush.fill_(float(i))
        a, b = ev(), ev()
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        tot += a.elapsed_time(b)
    return tot / reps


def run_extras(dev, flush, peak, step2d, x0, y, B):
    """The other configurations of this path, each timed on its own (one GPU)."""
    import torch
    import pridediff_gb300 as P
    ev = lambda: torch.cuda.Event(enable_timing=True)   # noqa: E731
    out = {}

    def frac(bytes_, ms):
        gbs = bytes_ / (ms / 1e3) / 1e9
        return {"achieved_GBps": gbs, "frac_of_measured_peak": gbs / peak}

    # plain single-instance GPU path: the same 16 slices one call at a time
    try:
        def plain():
            for i in range(B):
                step2d(x0[i:i + 1], y[i:i + 1])
        ms = _timed(plain, 3, flush, ev)
        out["plain_per_slice"] = {"what": "headline workload, one slice per autograd call (no batching, no graph)",
                                  "ms_per_step": ms, "value": B / (ms / 1e3), "unit": UNIT}
    except Exception as e:   # report, never hide the headline line
        out["plain_per_slice"] = {"error": repr(e)}

    # parallel beam, the reference's CPU-runnable configuration: one 256^2 slice
    # at 1 mm, 180 views over 180 degrees, 367 detectors of 1 mm; loss + backward
    try:
        projp = P.projector2d(256, 367, 1.0, 1.0, 500.0, 1000.0, scan_type="para").to(dev)
        angp = torch.arange(180, dtype=torch.float32, device=dev) * (np.pi / 180)
        xp = torch.from_numpy(phantom(256, 256, 10, np.random.default_rng(7), 1.0))[None, None].to(dev)
        with torch.no_grad():
            yp = projp.projection(xp, angp)

        def stepp():
            xr = (xp * 0.8).requires_grad_(True)
            ((projp.projection(xr, angp) - yp) ** 2).sum().backward()
        ms = _timed(stepp, 20, flush, ev)
        nbp = 2 * 4.0 * 180 * (256 * 256 + 367)
        out["para_1x256_180v"] = {"what": "parallel beam 256^2 at 1 mm, 180 views over 180 deg, 367 dets of 1 mm, "
                                          "one slice, loss + backward (launch-latency bound)",
                                  "ms_per_step": ms, "value": 1 / (ms / 1e3), "unit": UNIT, **frac(nbp, ms),
                                  "bytes_model": "view-swept 4*V*(H*W + D) per slice and operator"}
        del projp, xp, yp
    except Exception as e:   # report, never hide the headline line
        out["para_1x256_180v"] = {"error": repr(e)}

    # FBP (deeprecon's filtered_backprojection) of the headline sinograms
    try:
        ct = P._native.ctypes
        proj = P.projector2d(512, 736, 0.66, 1.2858, 595.0, 1085.6, scan_type="flat").to(dev)
        V = y.shape[2]
        ang = torch.arange(V, dtype=torch.float32, device=dev) * (2 * np.pi / V)
        with torch.no_grad():
            fbp = lambda: proj.filtered_backprojection(y, ang)   # noqa: E731

            def composed():   # the reference's composition: torch conv2d, then the weighted BP
                f = torch.nn.functional.conv2d(y * proj.weight, proj.filter, padding=(0, 735))
                return proj.backprojection_w(f, ang) * (ang[-1] - ang[0]).abs() / (V - 1) / 2

            ms = _timed(fbp, 3, flush, ev)
            ms_conv = _timed(composed, 3, flush, ev)
            lib = P._native.load()
            lib.dd_profile_enable(1)
            for _ in range(3):
                fbp()
            torch.cuda.synchronize()
            tot, cnt = ct.c_double(), ct.c_int()
            lib.dd_profile_read(4, ct.byref(tot), ct.byref(cnt))
            lib.dd_profile_enable(0)
        fms = tot.value / max(cnt.value, 1)
        flops = 2.0 * B * V * 736 * 736
        out["fbp_16x512_720v"] = {
            "what": "projector2d.filtered_backprojection of the 16 headline sinograms (cosine weight + ramp "
                    "filter fused in one kernel, then the weighted DD back-projection)",
            "ms_per_call": ms, "value": B / (ms / 1e3), "unit": "FBP/s",
            "ms_per_call_torch_conv2d_composition": ms_conv,
            "filter_kernel_ms": fms, "filter_kernel_TFLOPs_fp32": flops / (fms / 1e3) / 1e12}
    except Exception as e:
        out["fbp_16x512_720v"] = {"error": repr(e)}

    # batched uneven DC loop: 24 instances, 50 graph-captured steps, eta 1e-3
    try:
        from pridediff_gb300.batch import UnevenBatch2d
        from pridediff_gb300 import autotune
        rng = np.random.default_rng(2024)
        projs, angs, imgs, nbytes = [], [], [], 0.0
        for _ in range(24):
            n = int(rng.choice([256, 384, 512]))
            V = int(rng.choice([360, 576, 720]))
            D = int(rng.choice([368, 512, 736]))
            projs.append(P.projector2d(n, D, 0.66, 1.2858, 595.0, 1085.6, scan_type="flat").to(dev))
            angs.append(torch.arange(V, dtype=torch.float32, device=dev) * (2 * np.pi / V))
            imgs.append(torch.from_numpy(phantom(n, n, 10, rng, 0.04))[None, None].to(dev))
            nbytes += 2 * 4.0 * V * (n * n + D)
        ub = UnevenBatch2d(projs, angs)
        xt = ub.pack(imgs)
        yb = ub.forward(xt)
        xs = (xt * 0.8).contiguous()
        import tempfile
        tune = autotune.tune_batch_dc(ub, xs, yb, eta=0.0, reps=2,
                                      path=os.path.join(tempfile.gettempdir(), "pridediff_bench_tune.json"))
        steps = 50
        xg = xs.clone()
        graph = ub.dc_graph(xg, yb, 1e-3, steps)
        ms = _timed(lambda: graph.replay(), 3, flush, ev)
        xe = xs.clone()
        ms_eager = _timed(lambda: ub.dc_step(xe, yb, 1e-3), 3, flush, ev)
        out["batched_dc_24_uneven"] = {
            "what": "24 uneven fan-flat instances (image {256,384,512}^2, views {360,576,720}, dets "
                    "{368,512,736}), x <- x - 1e-3 A^T(Ax - y), 50 steps in one CUDA graph, one persistent "
                    "launch per operator, launch shape autotuned",
            "tune": tune, "ms_per_step": ms / steps, "ms_per_step_eager_no_graph": ms_eager,
            "value": 24 * steps / (ms / 1e3), "unit": UNIT, **frac(nbytes, ms / steps),
            "bytes_model": "view-swept 4*V*(H*W + D) per instance and operator, FP + BP per step"}
        del ub, graph, xg, xe, xs, yb, xt
    except Exception as e:
        out["batched_dc_24_uneven"] = {"error": repr(e)}
    torch.cuda.empty_cache()

    # 3-D cone-flat: 2 x 256^3, 360 views, 512 x 384 detector, autograd FP + BP
    try:
        proj = P.projector3d((256, 256, 256), (512, 384), 1.0, 1.0, 500.0, 1000.0, scan_type="flat").to(dev)
        ang = torch.arange(360, dtype=torch.float32, device=dev) * (2 * np.pi / 360)
        x3 = torch.stack([_ellipsoids((256, 256, 256), 12, 40 + i, 1.0, dev) for i in range(2)])[:, None]
        with torch.no_grad():
            y3 = proj.projection(x3, ang)

        def step3():
            xr = x3.detach().requires_grad_(True)
            ((proj.projection(xr, ang) - y3) ** 2).sum().backward()
        ms = _timed(step3, 3, flush, ev)
        nb3 = 2 * 2 * 4.0 * 360 * (256 ** 3 + 384 * 512)
        out["cone_flat_2x256^3"] = {"what": "cone-flat 2 x 256^3, 360 views, 512 x 384 detector, loss + backward",
                                    "ms_per_step": ms, "value": 2 / (ms / 1e3), "unit": UNIT, **frac(nb3, ms),
                                    "bytes_model": "view-swept 4*V*(W*H*D + R*C) per volume and operator"}
        del proj, x3, y3
    except Exception as e:
        out["cone_flat_2x256^3"] = {"error": repr(e)}
    torch.cuda.empty_cache()

    # 3-D spiral: 2 x 512x512x128, 3456 views, 64 x 736 arc detector, graph-captured DC steps
    try:
        import ctypes
        from pridediff_gb300 import _native as N
        from pridediff_gb300 import radontorch as RT
        V = 3456
        pitch = 1.0 * 64 * 1.0 * 595.0 / 1085.6 / 1152
        sp = torch.zeros((4, V), device=dev)
        sp[0] = -pitch * (V - 1) / 2 + pitch * torch.arange(V, device=dev, dtype=torch.float32)
        projs = P.projectorsp((512, 512, 128), (736, 64), (0.66, 0.66, 1.0), (1.2858, 1.0), 595.0, 1085.6).to(dev)
        ang = torch.arange(V, dtype=torch.float32, device=dev) * (2 * np.pi / 1152)
        x5 = torch.stack([_ellipsoids((128, 512, 512), 12, 60 + i, 0.04, dev) for i in range(2)])
        g5 = N.geom3d(RT.host_options(projs.options), spiral=True)
        lib = N.load()
        plan = RT.plan3d("spiral", g5, ang, sp)
        with torch.no_grad():
            y5 = projs.projection(x5[:, None], ang, sp)[:, 0].contiguous()
        nws = int(lib.dd3d_dc_workspace_bytes(2, g5, 2, V))
        ws = torch.empty(nws, dtype=torch.uint8, device=dev)
        resid = torch.empty_like(y5)
        xs5 = (x5 * 0.8).contiguous()
        steps = 5

        def dc():
            st = lib.dd3d_dc_step(2, g5, plan.data_ptr(), xs5.data_ptr(), y5.data_ptr(), resid.data_ptr(),
                                  ctypes.c_float(1e-3), 2, V, ws.data_ptr(), nws,
                                  torch.cuda.current_stream(dev).cuda_stream)
            if st != 0:
                raise RuntimeError(N.status_string(st))
        dc()
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(s):
            with torch.cuda.graph(graph, stream=s):
                for _ in range(steps):
                    dc()
        torch.cuda.current_stream(dev).wait_stream(s)
        ms = _timed(lambda: graph.replay(), 1, flush, ev) / steps
        zeff = 64 * 1.0 * 595.0 / 1085.6 / 1.0
        nb5 = 2 * 2 * 4.0 * V * (512 * 512 * zeff + 64 * 736)
        out["spiral_2x512x512x128"] = {
            "what": "spiral 2 x 512x512x128 (0.66 x 0.66 x 1.0 mm), 3456 views (3 turns, pitch 1), 64 x 736 arc "
                    "detector; DC steps x <- x - 1e-3 A^T(Ax - y), 5 steps in one CUDA graph (the configuration "
                    "runs 20)", "ms_per_step": ms, "value": 2 / (ms / 1e3), "unit": UNIT, **frac(nb5, ms),
            "bytes_model": "view-swept 4*V*(W*H*Z_eff + R*C), Z_eff = 35.08 slices, per volume and operator"}
        del graph, plan, ws, x5, xs5, y5, resid
    except Exception as e:
        out["spiral_2x512x512x128"] = {"error": repr(e)}
    torch.cuda.empty_cache()
    return out


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
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other configurations (batched DC loop, plain per-slice calls, 3-D)")
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
    from pridediff_gb300.replicas import max_over_ranks
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
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(starts, stops)) / args.steps, dev)
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
    compulsory = 4.0 * B * (512 * 512 + V * 736)         # image in + sinogram out (or back)

    # ---- end to end through the public API with host buffers: every step copies
    # its inputs in from pinned host memory and its gradient back out.  A copy
    # stream moves step i + 1's inputs (into the other of two device buffers)
    # and step i's gradient while the compute stream runs; the timed region runs
    # from before the first input copy to after the last gradient copy and
    # includes the L2 flush before every step.
    x_host = x0.detach().cpu().pin_memory()
    y_host = y.detach().cpu().pin_memory()
    g_host = torch.empty_like(x_host).pin_memory()
    xd = [torch.empty_like(x0) for _ in range(2)]
    yd = [torch.empty_like(y) for _ in range(2)]
    main = torch.cuda.current_stream(dev)
    cs = torch.cuda.Stream(dev)
    loaded = [torch.cuda.Event() for _ in range(2)]
    freed = [torch.cuda.Event() for _ in range(2)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def load(i):
        j = i % 2
        with torch.cuda.stream(cs):
            if i >= 2:
                cs.wait_event(freed[j])   # step i - 2 is done with these buffers
            xd[j].copy_(x_host, non_blocking=True)
            yd[j].copy_(y_host, non_blocking=True)
            loaded[j].record(cs)

    barrier()
    torch.cuda.synchronize()
    t_start.record(main)
    cs.wait_stream(main)
    load(0)
    for i in range(args.steps):
        j = i % 2
        if i + 1 < args.steps:
            load(i + 1)
        flush.fill_(float(i))
        main.wait_event(loaded[j])
        g, _ = step(xd[j], yd[j])
        freed[j].record(main)
        with torch.cuda.stream(cs):
            cs.wait_event(freed[j])
            g.record_stream(cs)
            g_host.copy_(g, non_blocking=True)
    main.wait_stream(cs)
    t_end.record(main)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(t_start.elapsed_time(t_end) / args.steps, dev)
    e2e_value = world * B / (e2e_ms / 1e3)

    extras = None
    if world == 1 and not args.no_extras:
        extras = run_extras(dev, flush, peak, step, x0, y, B)
        plain = extras.get("plain_per_slice", {}).get("value")
        if plain:
            extras["batched_over_plain"] = value / plain

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
                         "bytes_model": "view-swept 4*V*(H*W + D) per slice per operator",
                         # the compulsory bytes of one launch (inputs + outputs once) and the
                         # (view, pixel) incidences per second of the whole step
                         "compulsory_bytes_per_launch": compulsory,
                         "compulsory_frac": compulsory / (dom_ms / 1e3) / 1e9 / peak,
                         "incidences_per_s": 2.0 * world * B * V * 512 * 512 / (ms / 1e3)},
            "kernels": kern,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(x_host.numel() * 4 + y_host.numel() * 4),
                    "d2h_bytes_per_step": int(g_host.numel() * 4)},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "wall_s_timed_region": wall,
            "cpu_baseline": cpu,
        }
        if extras is not None:
            line["extra"] = extras
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

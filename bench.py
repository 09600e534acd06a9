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
  python bench.py --micro SCAN --op OP [--batch B] [--views V] [--size N] [--dets D] [--iters I]
                  [--impl ours|reference]

--micro repeats one operator on a bounded problem and prints its mean
CUDA-event time (the commands of the profiles/ summaries): SCAN is flat or
arc (the 512^2 fan geometry above; --size, --dets change it), para (1 mm
pixels and cells, views over 180 deg), --op fbp for filtered_backprojection, cone_flat or cone_arc (256^3, 512 x 384
detector, SID 500 / SDD 1000, --views of 360 angles over 360 deg), spiral
(512 x 512 x 128, 64 x 736 arc detector, the first --views views of the
comparator's middle turn) or uneven (the 24-instance uneven batch, one persistent launch
per call; --op proj or proj_t).  With --impl reference it times deeprecon's
own CUDA kernel for the same operator (built from the reference sources into
oracle/_ref/cuda where they exist).

On one GPU the line also carries `extra`: the same slices through the plain
per-slice path (the unbatched comparator), the parallel-beam configuration
(one 256^2 slice, 180 views, 367 detectors), the FBP of the 16 sinograms (fused
weight + filter kernel, then the weighted back-projection, beside the
reference's torch-convolution composition), the 24-instance uneven batched
data-consistency loop captured in a CUDA graph, and the 3-D cone-flat and
spiral configurations, each with its view-swept bytes against the measured
HBM peak.

--impl reference times deeprecon's CPU algorithm on this host on the same
workload, a bounded sample of slices per step: its own build where the
reference sources were compiled for this host (oracle/_ref), else the FP32
oracle port, which is bit-identical to it.
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


def _cpu_impl():
    """deeprecon's CPU fan-flat forward and adjoint on this host: its own build
    (oracle/_ref/libddref.so, compiled from the reference sources where they
    exist; an x86 build does not run on another host CPU) or else the FP32
    oracle port, which is bit-identical to it.  Both split the views over
    min(ceil(V / 128), cores) threads, the reference's own rule
    (FanFlatDisCPU2d.cpp:811-813)."""
    import oracle
    oracle.build()
    threads = oracle.default_threads(GEOM["views"])
    kind = "port"
    fwd = lambda x, a: oracle.run2d("flat", "proj", x, a, OPTIONS, "f", threads)     # noqa: E731
    adj = lambda r, a: oracle.run2d("flat", "proj_t", r, a, OPTIONS, "f", threads)   # noqa: E731
    if oracle.have_ref():
        try:
            z = np.zeros((1, 8, 8), np.float32)
            oracle.ref2d("flat", "proj", z, np.zeros(2, np.float32), [8, 8, 8, 1, 1, 1, 500, 1000, 0, 0, 0])
            kind = "reference"
            fwd = lambda x, a: oracle.ref2d("flat", "proj", x, a, OPTIONS)      # noqa: E731
            adj = lambda r, a: oracle.ref2d("flat", "proj_t", r, a, OPTIONS)    # noqa: E731
        except OSError:
            pass
    return kind, threads, fwd, adj


def cpu_port_baseline(seconds=10.0):
    """deeprecon's CPU algorithm on one slice at a time (see _cpu_impl)."""
    kind, threads, fwd, adj = _cpu_impl()
    rng = np.random.default_rng(99)
    ang = angles_np()
    img = phantom(512, 512, 10, rng, 0.04)[None]
    r = rng.standard_normal((1, GEOM["views"], GEOM["num_det"])).astype(np.float32)
    n = 0
    t0 = time.perf_counter()
    while True:
        fwd(img, ang)
        adj(r, ang)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": threads, "host_cpus": os.cpu_count(), "kind": kind,
            "sample": f"{n} slice(s) of the 16-slice workload, one at a time, forward + exact adjoint, "
                      f"{dt:.1f} s; FP+BP/s per slice, the unit of the GPU line"
                      + ("" if kind == "reference" else "; the port takes 1.27x the time of the reference's "
                         "own build on an x86 host (1.35 vs 1.07 s per slice, identical outputs)")}


def run_reference(args):
    """--impl reference: the CPU implementation on this host, same workload and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    kind, threads, fwd, adj = _cpu_impl()
    rng = np.random.default_rng(99)
    ang = angles_np()
    per_step = 1   # slices per step (bounded sample: one slice of the 16-slice batch)
    imgs = [phantom(512, 512, 10, rng, 0.04)[None] for _ in range(per_step)]
    r = rng.standard_normal((1, GEOM["views"], GEOM["num_det"])).astype(np.float32)

    def step():
        for im in imgs:
            fwd(im, ang)
            adj(r, ang)

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
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "host_cpus": os.cpu_count(),
                             "kind": kind,
                             "sample": f"{per_step} slice of the 16-slice workload per step (forward + exact "
                                       "adjoint); FP+BP/s per slice, the unit of the GPU line"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    try:
        line["extra"] = {"reference_cuda": reference_cuda_extra()}
    except Exception as e:   # report, never hide the reference line
        line["extra"] = {"reference_cuda": {"error": repr(e)}}
    print(json.dumps(line))


def reference_cuda_extra():
    """deeprecon's own CUDA operators on this host's GPU (the plain-GPU
    comparator): the workloads of run_comparator_workloads, each step through
    its CUDA kernels compiled unmodified from the reference sources
    (oracle/_ref/cuda; absent where those sources were not available)."""
    import torch
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device on this host"}
    from oracle import refcuda
    if not refcuda.available():
        return {"unavailable": "reference CUDA fatbins absent (built only where the reference sources exist)"}
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)   # noqa: E731
    res = run_comparator_workloads(dev, flush, ev, refcuda.run)
    res["what"] = ("deeprecon's CUDA Proj + ProjTrans per loss + backward step, called as radontorch calls "
                   "them (options read by .item(), per-call texture staging); views where its walk start "
                   "ties index -1 within rounding are left out (4 cone-beam, 12 spiral)")
    return res


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
        projs, angs, imgs, nbytes = uneven_instances(dev)
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

    # the workloads of the plain-GPU comparator (deeprecon's own CUDA kernels,
    # timed by --impl reference), here through this library
    try:
        out["same_workloads_as_reference_cuda"] = run_comparator_workloads(dev, flush, ev, None)
    except Exception as e:
        out["same_workloads_as_reference_cuda"] = {"error": repr(e)}
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


def _micro_problem(args, dev):
    """(geometry, options, input, angles, source_pos) of a --micro run."""
    import torch
    import cases3d
    g = torch.Generator(device=dev).manual_seed(0)
    image_in = args.op in ("proj", "bproj_t", "bproj_tw")
    if args.micro in ("para", "flat", "arc"):
        n, D = args.size or 512, args.dets or 736
        if args.micro == "para":   # the parallel-beam configuration: 1 mm pixels and cells, 180 deg
            opt = [n, n, D, 1.0, 1.0, 1.0, 500.0, 1000.0, 0.0, 0.0, 0.0]
            ang = torch.arange(args.views, dtype=torch.float32, device=dev) * (np.pi / args.views)
        else:
            det = 1.2858 / 1085.6 if args.micro == "arc" else 1.2858
            opt = [n, n, D, 0.66, 0.66, det, 595.0, 1085.6, 0.0, 0.0, 0.0]
            ang = torch.arange(args.views, dtype=torch.float32, device=dev) * (2 * np.pi / args.views)
        shape = (args.batch, 1, n, n) if image_in else (args.batch, 1, args.views, D)
        return opt, torch.rand(shape, device=dev, generator=g), ang, None
    if args.micro in ("cone_flat", "cone_arc"):
        col = 1.0 / 1000.0 if args.micro == "cone_arc" else 1.0
        opt = [256, 256, 256, 512, 384, 1.0, 1.0, 1.0, col, 1.0, 500.0, 1000.0, 0, 0, 0, 0, 0]
        ang = torch.arange(args.views, dtype=torch.float32, device=dev) * (2 * np.pi / args.views)
        shape = (args.batch, 1, 256, 256, 256) if image_in else (args.batch, 1, args.views, 384, 512)
        return opt, torch.rand(shape, device=dev, generator=g), ang, None
    opt, ang_np, sp_np = cases3d.spiral_512x128()
    sel = comparator_views()[1][:args.views]   # views of the middle turn
    ang = torch.from_numpy(ang_np[sel].copy()).to(dev)
    sp = torch.from_numpy(sp_np[:, sel].copy()).to(dev)
    shape = (args.batch, 1, 128, 512, 512) if image_in else (args.batch, 1, args.views, 64, 736)
    return list(opt), torch.rand(shape, device=dev, generator=g) * 0.04, ang, sp


def run_micro(args):
    """--micro: `iters` applications of one operator, mean CUDA-event ms."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    dev = torch.device("cuda:0")
    if args.micro == "uneven":
        return run_micro_uneven(args, dev)
    if args.op == "fbp":
        return run_micro_fbp(args, dev)
    geo = {"para": "Para", "flat": "FanFlat", "arc": "FanArc", "cone_flat": "ConeFlat", "cone_arc": "ConeArc",
           "spiral": "Spiral"}[args.micro]
    dim = "2d" if args.micro in ("para", "flat", "arc") else "3d"
    name = {"proj": "Proj", "proj_t": "ProjTrans", "bproj": "BackProj", "bproj_t": "BackProjTrans",
            "bproj_w": "BackProjWeighted", "bproj_tw": "BackProjTransWeighted"}[args.op] + f"{geo}Dis{dim}"
    opt, x, ang, sp = _micro_problem(args, dev)
    if args.impl == "reference":
        import oracle
        from oracle import refcuda
        bad = oracle.scan_hazards(args.micro, ang.cpu().numpy(), opt,
                                  None if sp is None else sp.cpu().numpy()).sum()
        if bad:
            raise SystemExit(f"reference kernels not run: {bad} walk starts within rounding of index -1")
        ot = torch.tensor(opt, dtype=torch.float32)
        fn = lambda: refcuda.run(args.micro, args.op, x, ang, ot, sp)   # noqa: E731
        name = "deeprecon CUDA " + name
    else:
        from pridediff_gb300 import radontorch
        f = getattr(radontorch, name)
        ot = torch.tensor(opt, dtype=torch.float32)
        fn = (lambda: f(x, ot, ang, sp)) if sp is not None else (lambda: f(x, ot, ang))
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.iters):
        fn()
    b.record()
    torch.cuda.synchronize()
    print(f"{name} batch {args.batch}, {int(ang.numel())} views: {a.elapsed_time(b) / args.iters:.3f} ms per call")


def run_micro_fbp(args, dev):
    """--micro flat|arc|para --op fbp: projector2d.filtered_backprojection
    (fused weight + filter kernel, then the weighted DD back-projection)."""
    import torch
    import pridediff_gb300 as P
    n, D = args.size or 512, args.dets or 736
    pix, det = (1.0, 1.0) if args.micro == "para" else (0.66, 1.2858)
    proj = P.projector2d(n, D, pix, det, 595.0, 1085.6, scan_type=args.micro).to(dev)
    span = np.pi if args.micro == "para" else 2 * np.pi
    ang = torch.arange(args.views, dtype=torch.float32, device=dev) * (span / args.views)
    y = torch.rand((args.batch, 1, args.views, D), device=dev, generator=torch.Generator(device=dev).manual_seed(0))
    with torch.no_grad():
        fn = lambda: proj.filtered_backprojection(y, ang)   # noqa: E731
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.iters):
            fn()
        b.record()
        torch.cuda.synchronize()
    print(f"filtered_backprojection {args.micro} batch {args.batch}, {args.views} views: "
          f"{a.elapsed_time(b) / args.iters:.3f} ms per call")


def uneven_instances(dev, seed=2024, n=24):
    """The uneven batched configuration: n fan-flat instances with image size,
    view count and detector count drawn from {256,384,512}^2 x {360,576,720} x
    {368,512,736}, each with a seeded ellipse phantom."""
    import torch
    import pridediff_gb300 as P
    rng = np.random.default_rng(seed)
    projs, angs, imgs, nbytes = [], [], [], 0.0
    for _ in range(n):
        size = int(rng.choice([256, 384, 512]))
        V = int(rng.choice([360, 576, 720]))
        D = int(rng.choice([368, 512, 736]))
        projs.append(P.projector2d(size, D, 0.66, 1.2858, 595.0, 1085.6, scan_type="flat").to(dev))
        angs.append(torch.arange(V, dtype=torch.float32, device=dev) * (2 * np.pi / V))
        imgs.append(torch.from_numpy(phantom(size, size, 10, rng, 0.04))[None, None].to(dev))
        nbytes += 2 * 4.0 * V * (size * size + D)
    return projs, angs, imgs, nbytes


def run_micro_uneven(args, dev):
    import torch
    from pridediff_gb300.batch import UnevenBatch2d
    projs, angs, imgs, _ = uneven_instances(dev)
    ub = UnevenBatch2d(projs, angs)
    x = ub.pack(imgs)
    if args.op == "proj_t":
        x = ub.forward(x)
    fn = (lambda: ub.forward(x)) if args.op == "proj" else (lambda: ub.adjoint(x))
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.iters):
        fn()
    b.record()
    torch.cuda.synchronize()
    print(f"uneven batch of 24 {args.op}: {a.elapsed_time(b) / args.iters:.3f} ms per call")


# Views of the 3-D configurations that deeprecon's CUDA kernels are not run
# on: on these an image edge ties the first column boundary of a 256-column
# block to within rounding, where the reference's walk could start at index
# -1 and read or write out of bounds (tests/test_oracle.py checks these lists
# against the oracle's start-index scan).  Both sides of the comparator skip
# them.
CONE_REF_SKIP = [12, 102, 168, 258]
SPIRAL_TURN = (1152, 2304)   # the middle of the three turns
SPIRAL_REF_SKIP = [1267, 1333, 1339, 1555, 1613, 1829, 1835, 1901, 2117, 2123, 2197, 2203]


def comparator_views():
    """(cone-beam view indices, spiral view indices) of the comparator."""
    cone = np.setdiff1d(np.arange(360), CONE_REF_SKIP)
    spiral = np.setdiff1d(np.arange(*SPIRAL_TURN), SPIRAL_REF_SKIP)
    return cone, spiral


def run_comparator_workloads(dev, flush, ev, ref):
    """One loss + backward step (forward A x, residual, exact adjoint) on the
    headline fan-flat slices, on 2 x 256^3 cone-beam volumes (356 views) and
    on 2 x 512x512x128 spiral volumes (the middle turn's 1140 views).

    ref=None runs this library's projector modules (autograd).  Otherwise
    `ref` is deeprecon's CUDA operator (oracle/refcuda.run), called the way
    radontorch calls it (RadonTorch.cpp:17-83): eleven .item() reads of the
    device options (RadonTorch.cpp:19-29), an output from torch::empty or
    torch::zeros, and for the image-reading operators a cudaArray and texture
    built and freed around the launch (FanFlatDisCUDA2d.cu:777-815)."""
    import torch
    import pridediff_gb300 as P
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases3d
    res = {}
    B = GEOM["batch"]
    rng = np.random.default_rng(1234)
    x2 = torch.from_numpy(np.stack([phantom(512, 512, 10, rng, 0.04) for _ in range(B)])[:, None]).to(dev)
    y2 = torch.from_numpy(rng.random((B, 1, GEOM["views"], GEOM["num_det"]), dtype=np.float32) * 8.0).to(dev)
    ang2 = torch.from_numpy(angles_np()).to(dev)
    cone_v, spiral_v = comparator_views()
    o4, a4 = cases3d.cone_256cube()
    ang4 = torch.from_numpy(a4[cone_v].copy()).to(dev)
    x4 = torch.stack([_ellipsoids((256, 256, 256), 12, 40 + i, 1.0, dev) for i in range(2)])[:, None]
    y4 = torch.rand((2, 1, cone_v.size, 384, 512), device=dev) * 100.0
    o5, a5, s5 = cases3d.spiral_512x128()
    ang5 = torch.from_numpy(a5[spiral_v].copy()).to(dev)
    sp5 = torch.from_numpy(s5[:, spiral_v].copy()).to(dev)
    x5 = torch.stack([_ellipsoids((128, 512, 512), 12, 60 + i, 0.04, dev) for i in range(2)])[:, None]
    y5 = torch.rand((2, 1, spiral_v.size, 64, 736), device=dev) * 8.0

    if ref is None:
        p2 = P.projector2d(512, 736, 0.66, 1.2858, 595.0, 1085.6, scan_type="flat").to(dev)
        p4 = P.projector3d((256, 256, 256), (512, 384), 1.0, 1.0, 500.0, 1000.0, scan_type="flat").to(dev)
        p5 = P.projectorsp((512, 512, 128), (736, 64), (0.66, 0.66, 1.0), (1.2858, 1.0), 595.0, 1085.6).to(dev)

        def step(proj, x, yy, ang, sp=None):
            xr = x.detach().requires_grad_(True)
            fp = proj.projection(xr, ang, sp) if sp is not None else proj.projection(xr, ang)
            ((fp - yy) ** 2).sum().backward()
        s2 = lambda: step(p2, x2, y2, ang2)                               # noqa: E731
        s2_slice = lambda: [step(p2, x2[i:i + 1], y2[i:i + 1], ang2) for i in range(B)]   # noqa: E731
        s4 = lambda: step(p4, x4, y4, ang4)                               # noqa: E731
        s5 = lambda: step(p5, x5, y5, ang5, sp5)                          # noqa: E731
    else:
        opt2 = torch.tensor(OPTIONS, dtype=torch.float32, device=dev)
        opt4 = torch.tensor(o4, device=dev)
        opt5 = torch.tensor(o5, device=dev)

        def step(geom, opt, x, yy, ang, sp=None):
            fp = ref(geom, "proj", x, ang, [o.item() for o in opt], sp)
            ref(geom, "proj_t", 2.0 * (fp - yy), ang, [o.item() for o in opt], sp)
        s2 = lambda: step("flat", opt2, x2, y2, ang2)                     # noqa: E731
        s2_slice = lambda: [step("flat", opt2, x2[i:i + 1], y2[i:i + 1], ang2) for i in range(B)]   # noqa: E731
        s4 = lambda: step("cone_flat", opt4, x4, y4, ang4)                # noqa: E731
        s5 = lambda: step("spiral", opt5, x5, y5, ang5, sp5)              # noqa: E731

    ms = _timed(s2, 3, flush, ev)
    ms_slice = _timed(s2_slice, 3, flush, ev)
    res["fan_flat_16x512_720v"] = {"ms_per_step_16_slices_per_call": ms, "value_16_slices_per_call": B / (ms / 1e3),
                                   "ms_per_step_one_slice_per_call": ms_slice,
                                   "value_one_slice_per_call": B / (ms_slice / 1e3), "unit": UNIT}
    ms = _timed(s4, 2, flush, ev)
    res["cone_flat_2x256^3_356v"] = {"ms_per_step": ms, "value": 2 / (ms / 1e3), "unit": UNIT,
                                     "views": int(cone_v.size)}
    ms = _timed(s5, 1, flush, ev)
    res["spiral_2x512x512x128_1140v"] = {"ms_per_step": ms, "value": 2 / (ms / 1e3), "unit": UNIT,
                                         "views": int(spiral_v.size)}
    return res


def _forward_tune_record(lib):
    """The single-geometry forward shapes the autotuner chose in this run,
    with the CTA shape each resolves to (slices per CTA, cluster size)."""
    from pridediff_gb300 import autotune
    from pridediff_gb300 import _native as N
    out = []
    for rec in autotune.chosen():
        w, h = rec.get("image", [512, 512])
        g = N.Geom2d(w, h, rec.get("dets", 736), 0.66, 0.66, 1.2858, 595.0, 1085.6, 0.0, 0.0, 0.0)
        t = N.Tune2d()
        t.fwd_slices = int(rec["choice"].get("fwd_slices", 0))
        t.fwd_cluster = int(rec["choice"].get("fwd_cluster", 0))
        sl, cl = N.ctypes.c_int(), N.ctypes.c_int()
        lib.dd2d_fwd_shape(N.SCAN2D.get(rec.get("scan", "flat"), 1), g, t, N.ctypes.byref(sl), N.ctypes.byref(cl))
        out.append({**rec, "slices_per_cta": sl.value, "ctas_per_view_cluster": cl.value})
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
    ap.add_argument("--micro", default=None,
                    choices=["para", "flat", "arc", "cone_flat", "cone_arc", "spiral", "uneven"],
                    help="time one operator on a bounded problem instead (see the module docstring)")
    ap.add_argument("--op", default="proj",
                    choices=["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw", "fbp"])
    ap.add_argument("--size", type=int, default=0, help="--micro 2-D: image size (default 512)")
    ap.add_argument("--dets", type=int, default=0, help="--micro 2-D: detector cells (default 736)")
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--views", type=int, default=720)
    ap.add_argument("--iters", type=int, default=3)
    args = ap.parse_args()
    if args.micro:
        run_micro(args)
        return
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
            "tune": {"forward2d": _forward_tune_record(lib)},
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

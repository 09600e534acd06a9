"""Kernel microbenchmark: repeat one operator on a bounded problem.

    python -m pridediff_gb300.microbench --scan flat --op proj --batch 8 --iters 3
    python -m pridediff_gb300.microbench --scan cone_flat --op proj_t --batch 2 --views 36 --iters 2

2-D (para / flat / arc): the 16-slice fan geometry (512^2 at 0.66 mm, 736
detectors of 1.2858 mm, SID 595, SDD 1085.6).  3-D cone_flat / cone_arc: the
cone-beam configuration (256^3 at 1 mm, 512 x 384 detector of 1 mm cells,
SID 500, SDD 1000), --views of its 360 view angles spaced over 360 degrees.

Runs `iters` applications of one radontorch operator on seeded data (the
geometry plan is built before the loop) and prints the mean CUDA-event time.
Used for profiler captures of a single kernel on a bounded problem.
"""
from __future__ import annotations

import argparse

import numpy as np
import torch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--scan", default="flat", choices=["para", "flat", "arc", "cone_flat", "cone_arc"])
    ap.add_argument("--op", default="proj", choices=["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"])
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--views", type=int, default=720)
    ap.add_argument("--dets", type=int, default=736)
    ap.add_argument("--iters", type=int, default=3)
    args = ap.parse_args(argv)
    from . import radontorch
    if args.scan.startswith("cone"):
        return main3d(args)
    geo = {"para": "Para", "flat": "FanFlat", "arc": "FanArc"}[args.scan]
    name = {"proj": "Proj{}Dis2d", "proj_t": "ProjTrans{}Dis2d", "bproj": "BackProj{}Dis2d",
            "bproj_t": "BackProjTrans{}Dis2d", "bproj_w": "BackProjWeighted{}Dis2d",
            "bproj_tw": "BackProjTransWeighted{}Dis2d"}[args.op].format(geo)
    fn = getattr(radontorch, name)
    det = 1.2858 / 1085.6 if args.scan == "arc" else 1.2858
    opt = torch.tensor([args.size, args.size, args.dets, 0.66, 0.66, det, 595.0, 1085.6, 0.0, 0.0, 0.0])
    dev = torch.device("cuda:0")
    ang = torch.arange(args.views, dtype=torch.float32, device=dev) * (2 * np.pi / args.views)
    g = torch.Generator(device=dev).manual_seed(0)
    if args.op in ("proj", "bproj_t", "bproj_tw"):
        x = torch.rand((args.batch, 1, args.size, args.size), device=dev, generator=g)
    else:
        x = torch.randn((args.batch, 1, args.views, args.dets), device=dev, generator=g)
    fn(x, opt, ang)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.iters):
        fn(x, opt, ang)
    b.record()
    torch.cuda.synchronize()
    print(f"{name} batch {args.batch}: {a.elapsed_time(b) / args.iters:.3f} ms per call")


def main3d(args):
    from . import radontorch
    geo = {"cone_flat": "ConeFlat", "cone_arc": "ConeArc"}[args.scan]
    name = {"proj": "Proj{}Dis3d", "proj_t": "ProjTrans{}Dis3d", "bproj": "BackProj{}Dis3d",
            "bproj_t": "BackProjTrans{}Dis3d", "bproj_w": "BackProjWeighted{}Dis3d",
            "bproj_tw": "BackProjTransWeighted{}Dis3d"}[args.op].format(geo)
    fn = getattr(radontorch, name)
    col = 1.0 / 1000.0 if args.scan == "cone_arc" else 1.0
    opt = torch.tensor([256, 256, 256, 512, 384, 1.0, 1.0, 1.0, col, 1.0, 500.0, 1000.0, 0, 0, 0, 0, 0],
                       dtype=torch.float32)
    dev = torch.device("cuda:0")
    ang = torch.arange(args.views, dtype=torch.float32, device=dev) * (2 * np.pi / args.views)
    g = torch.Generator(device=dev).manual_seed(0)
    if args.op in ("proj", "bproj_t", "bproj_tw"):
        x = torch.rand((args.batch, 1, 256, 256, 256), device=dev, generator=g)
    else:
        x = torch.rand((args.batch, 1, args.views, 384, 512), device=dev, generator=g)
    fn(x, opt, ang)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.iters):
        fn(x, opt, ang)
    b.record()
    torch.cuda.synchronize()
    print(f"{name} batch {args.batch}, {args.views} views: {a.elapsed_time(b) / args.iters:.3f} ms per call")


if __name__ == "__main__":
    main()

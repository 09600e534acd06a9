"""Generate the golden vectors under tests/golden/ from deeprecon's own CPU code.

Run in a checkout where the reference sources exist (they are compiled into
oracle/_ref/libddref.so by `make -C oracle`):

    python tests/golden/make_golden.py               # operator outputs -> dd2d_golden.npz
    python tests/golden/make_golden.py --sysmatrix   # system matrices  -> sysmat_golden.npz
    python tests/golden/make_golden.py --fbp         # FBP              -> fbp_golden.npz
    python tests/golden/make_golden.py --cuda3d [--out PATH]   # 3-D -> dd3d_golden.npz

The --cuda3d mode runs deeprecon's own CUDA kernels (the reference for the
3-D geometries, which have no CPU path) and so needs a GPU and the fatbins
that `make -C oracle` compiles from the reference sources (oracle/refcuda.py).

Every case stores its seeded inputs and the reference outputs (computed by
the unmodified deeprecon CPU projectors, single-threaded), so the tests can
check the oracle and the CUDA path on machines where the reference cannot be
built.  Cases are small (tens of KB each).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

OPS2D = {"para": ["proj", "proj_t", "bproj", "bproj_t"],
         "flat": ["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"],
         "arc": ["proj", "proj_t", "bproj", "bproj_t", "bproj_w", "bproj_tw"]}

# (name, geometry, options, angles): odd sizes, shifts and non-square pixels
CASES = [
    ("para_small", "para", [64, 48, 95, 1.0, 1.1, 1.0, 500.0, 1000.0, 0.3, -0.2, 0.25],
     np.arange(90) * np.pi / 90),
    ("flat_small", "flat", [64, 48, 80, 0.9, 0.8, 1.3, 595.0, 1085.6, 0.5, -0.4, 0.6],
     np.arange(120) * 2 * np.pi / 120),
    ("arc_small", "arc", [64, 48, 80, 0.9, 0.8, 1.3 / 1085.6, 595.0, 1085.6, 0.5, -0.4, 0.6 / 1085.6],
     np.arange(120) * 2 * np.pi / 120),
    ("flat_odd", "flat", [37, 53, 61, 1.7, 1.3, 2.1, 400.0, 800.0, -1.2, 0.7, -0.9],
     np.linspace(0.1, 6.0, 47)),
]


def ellipse_phantom(h, w, n, rng, scale=1.0):
    """Additive ellipses at pixel centres (the convention of deeprecon's phantom.py)."""
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    cy, cx = (h - 1) / 2.0, (w - 1) / 2.0
    img = np.zeros((h, w))
    for _ in range(n):
        x0 = rng.uniform(-0.8, 0.8) * w / 2 + cx
        y0 = rng.uniform(-0.8, 0.8) * h / 2 + cy
        a, b = rng.uniform(2, max(3, w / 4)), rng.uniform(2, max(3, h / 4))
        t = rng.uniform(0, np.pi)
        dx, dy = xx - x0, yy - y0
        u = dx * np.cos(t) + dy * np.sin(t)
        v = -dx * np.sin(t) + dy * np.cos(t)
        img[(u / a) ** 2 + (v / b) ** 2 <= 1] += rng.uniform(0, 1) * scale
    return img.astype(np.float32)


def main():
    if not oracle.have_ref():
        oracle.build()
    if not oracle.have_ref():
        raise SystemExit("reference sources not present: cannot regenerate golden vectors")
    out = {}
    for seed, (name, geom, opt, ang) in enumerate(CASES):
        rng = np.random.default_rng(1000 + seed)
        ang = ang.astype(np.float32)
        W, H, D = opt[0], opt[1], opt[2]
        img = np.stack([ellipse_phantom(H, W, 6, rng), rng.random((H, W)).astype(np.float32)])
        sino = rng.standard_normal((2, len(ang), D)).astype(np.float32)
        out[f"{name}/options"] = np.asarray(opt, np.float32)
        out[f"{name}/angles"] = ang
        out[f"{name}/image"] = img
        out[f"{name}/sino"] = sino
        for op in OPS2D[geom]:
            x = img if op in oracle.IMAGE_INPUT else sino
            out[f"{name}/{op}/ref"] = oracle.ref2d(geom, op, x, ang, opt)
    path = os.path.join(HERE, "dd2d_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KB")


# (name, geometry, options, angles) for the system matrices: small images so
# that each COO matrix stays at a few thousand entries; views include the
# 45-degree branch boundary and flipped detectors
SYS_CASES = [
    ("para_sys", "para", [20, 16, 27, 1.0, 1.1, 1.0, 500.0, 1000.0, 0.3, -0.2, 0.25],
     np.concatenate([np.arange(10) * np.pi / 10, [np.pi / 4]])),
    ("flat_sys", "flat", [20, 16, 25, 0.9, 0.8, 1.3, 595.0, 1085.6, 0.5, -0.4, 0.6],
     np.concatenate([np.arange(12) * 2 * np.pi / 12, [np.pi / 4, 3 * np.pi / 4]])),
    ("arc_sys", "arc", [20, 16, 25, 0.9, 0.8, 1.3 / 1085.6, 595.0, 1085.6, 0.5, -0.4, 0.6 / 1085.6],
     np.concatenate([np.arange(12) * 2 * np.pi / 12, [np.pi / 4, 3 * np.pi / 4]])),
]


def main_sysmatrix():
    """deeprecon's GetSysMatrix* COO matrices (rows, cols, vals in its order)."""
    if not oracle.have_ref():
        oracle.build()
    if not oracle.have_ref():
        raise SystemExit("reference sources not present: cannot regenerate golden vectors")
    out = {}
    for name, geom, opt, ang in SYS_CASES:
        ang = np.asarray(ang, np.float32)
        rows, cols, vals = oracle.ref_sysmatrix(geom, ang, opt)
        out[f"{name}/options"] = np.asarray(opt, np.float32)
        out[f"{name}/angles"] = ang
        out[f"{name}/rows"] = rows
        out[f"{name}/cols"] = cols
        out[f"{name}/vals"] = vals
    path = os.path.join(HERE, "sysmat_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KB")


# (name, geometry, projector2d arguments, angles, filter_type, redundant)
FBP_CASES = [
    ("flat_fbp", "flat", dict(image_size=(64, 48), num_det=80, pix_size=(0.9, 0.8), det_size=1.3,
                              iso_source=595.0, source_detector=1085.6, pixshift=(0.5, -0.4), binshift=0.6),
     np.arange(120) * 2 * np.pi / 120, "ramp", True),
    ("arc_fbp", "arc", dict(image_size=(64, 48), num_det=80, pix_size=(0.9, 0.8), det_size=1.3,
                            iso_source=595.0, source_detector=1085.6, pixshift=(0.5, -0.4), binshift=0.6),
     np.arange(120) * 2 * np.pi / 120, "sheeplogan", True),
    ("para_fbp", "para", dict(image_size=(64, 48), num_det=95, pix_size=(1.0, 1.1), det_size=1.0,
                              iso_source=500.0, source_detector=1000.0, pixshift=(0.3, -0.2), binshift=0.25),
     np.arange(90) * np.pi / 90, "ramp", False),
]


def _reference_projector_module():
    """deeprecon's own deeprecon.torch.projector package, imported from the
    reference sources with its compiled `radontorch` extension answered by the
    reference's CPU projectors (oracle/_ref/libddref.so): the Python code that
    runs -- weights, filters, the convolution, the scaling -- is the
    reference's, unmodified."""
    import importlib.util
    import types

    import torch
    stub = types.ModuleType("radontorch")
    ops = {"Proj": "proj", "ProjTrans": "proj_t", "BackProj": "bproj", "BackProjTrans": "bproj_t",
           "BackProjWeighted": "bproj_w", "BackProjTransWeighted": "bproj_tw"}
    geoms = {"Para": "para", "FanFlat": "flat", "FanArc": "arc"}

    def make(geom, op):
        def f(x, options, angles):
            y = oracle.ref2d(geom, op, x.detach().cpu().numpy()[:, 0], angles.detach().cpu().numpy(),
                             options.detach().cpu().numpy())
            return torch.from_numpy(np.ascontiguousarray(y, dtype=np.float32))[:, None]
        return f

    for on, o in ops.items():
        for gn, g in geoms.items():
            setattr(stub, f"{on}{gn}Dis2d", make(g, o))
    sys.modules["radontorch"] = stub
    ref = os.environ.get("REF", "/root/reference/deeprecon")
    pkg = os.path.join(ref, "deeprecon", "torch", "projector")
    spec = importlib.util.spec_from_file_location("ref_projector", os.path.join(pkg, "__init__.py"),
                                                  submodule_search_locations=[pkg])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ref_projector"] = mod
    spec.loader.exec_module(mod)
    return mod


def main_fbp():
    """deeprecon's projector2d.filtered_backprojection, its filter taps and
    cosine weights."""
    import torch
    if not oracle.have_ref():
        oracle.build()
    if not oracle.have_ref():
        raise SystemExit("reference sources not present: cannot regenerate golden vectors")
    refp = _reference_projector_module()
    out = {}
    for seed, (name, geom, kw, ang, ftype, redundant) in enumerate(FBP_CASES):
        rng = np.random.default_rng(2000 + seed)
        ang = np.asarray(ang, np.float32)
        prj = refp.projector2d(scan_type=geom, filter_type=ftype, **kw)
        W, H = kw["image_size"]
        img = ellipse_phantom(H, W, 6, rng)[None]
        x = torch.from_numpy(img)[:, None]
        sino = prj.projection(x, torch.from_numpy(ang))
        rec = prj.filtered_backprojection(sino, torch.from_numpy(ang), redundant=redundant)
        out[f"{name}/options"] = prj.options.detach().numpy()
        out[f"{name}/ctor"] = np.asarray([W, H, kw["num_det"], *kw["pix_size"], kw["det_size"], kw["iso_source"],
                                          kw["source_detector"], *kw["pixshift"], kw["binshift"]], np.float64)
        out[f"{name}/angles"] = ang
        out[f"{name}/sino"] = sino.numpy()[:, 0]
        out[f"{name}/filter"] = prj.filter.detach().numpy().reshape(-1)
        out[f"{name}/weight"] = prj.weight.detach().numpy()
        out[f"{name}/fbp"] = rec.numpy()[:, 0]
        for other in ("ramp", "sheeplogan"):
            out[f"{name}/taps_{other}"] = prj.filter_generate(other).detach().numpy().reshape(-1)
    path = os.path.join(HERE, "fbp_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KB")


def main_cuda3d(path):
    """deeprecon's CUDA outputs for the 18 3-D operators on the small cases of
    tests/cases3d.py (batch 1, inputs from cases3d.inputs(seed=31)), and for
    Proj / ProjTrans on view subsets of the full cone-beam and spiral
    configurations (outputs subsampled by the strides in cases3d)."""
    import torch

    sys.path.insert(0, os.path.dirname(HERE))
    import cases3d
    from oracle import refcuda
    if not refcuda.available():
        raise SystemExit("reference CUDA fatbins absent: run make -C oracle where the reference sources exist")
    dev = torch.device("cuda:0")

    def ref(geom, op, x, ang, opt, sp=None):
        assert oracle.scan_hazards(geom, ang, opt, sp).sum() == 0, (geom, op)
        xt = torch.from_numpy(np.ascontiguousarray(x, np.float32))[:, None].to(dev)
        at = torch.from_numpy(np.ascontiguousarray(ang, np.float32)).to(dev)
        st = None if sp is None else torch.from_numpy(np.ascontiguousarray(sp, np.float32)).to(dev)
        y = refcuda.run(geom, op, xt, at, opt, st)
        torch.cuda.synchronize()
        return y[:, 0].cpu().numpy()

    out = {}
    for name, case in sorted(cases3d.cases().items()):
        geom, opt, ang, sp = case
        x, y = cases3d.inputs(case, batch=1, seed=31)
        out[f"{name}/options"] = opt
        out[f"{name}/angles"] = ang
        if sp is not None:
            out[f"{name}/source_pos"] = sp
        for op in cases3d.OPS:
            out[f"{name}/{op}/ref"] = ref(geom, op, x if op in cases3d.IMAGE_IN else y, ang, opt, sp)

    opt, ang = cases3d.cone_256cube()
    sel = cases3d.CONE_VIEWS
    x = cases3d.ellipsoids(256, 256, 256, 12, 4)[None]
    yv = np.random.default_rng(5).random((1, sel.size, 384, 512)).astype(np.float32)
    out["cone256/x_sum"] = np.float64(x.sum(dtype=np.float64))
    out["cone256/proj/ref"] = ref("cone_flat", "proj", x, ang[sel], opt)[cases3d.CONE_SINO_STRIDE]
    out["cone256/proj_t/ref"] = ref("cone_flat", "proj_t", yv, ang[sel], opt)[cases3d.CONE_VOL_STRIDE]

    opt, ang, sp = cases3d.spiral_512x128()
    sel = cases3d.SPIRAL_VIEWS
    x = cases3d.ellipsoids(128, 512, 512, 12, 6, 0.04)[None]
    yv = np.random.default_rng(7).random((1, sel.size, 64, 736)).astype(np.float32)
    out["spiral512/x_sum"] = np.float64(x.sum(dtype=np.float64))
    out["spiral512/proj/ref"] = ref("spiral", "proj", x, ang[sel], opt, sp[:, sel])[cases3d.SPIRAL_SINO_STRIDE]
    out["spiral512/proj_t/ref"] = ref("spiral", "proj_t", yv, ang[sel], opt, sp[:, sel])[cases3d.SPIRAL_VOL_STRIDE]
    out["device"] = np.array(torch.cuda.get_device_name(0))
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KB")


if __name__ == "__main__":
    if "--cuda3d" in sys.argv[1:]:
        args = sys.argv[1:]
        main_cuda3d(args[args.index("--out") + 1] if "--out" in args else os.path.join(HERE, "dd3d_golden.npz"))
    elif "--sysmatrix" in sys.argv[1:]:
        main_sysmatrix()
    elif "--fbp" in sys.argv[1:]:
        main_fbp()
    else:
        main()

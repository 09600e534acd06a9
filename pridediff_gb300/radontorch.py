"""Drop-in for deeprecon's ``radontorch`` extension module.

Exposes the same 39 functions with the same tensor semantics as the pybind
module in deeprecon/interface/RadonTorch.cpp:1375-1418:

* ``Op(input, options, angles[, source_pos]) -> Tensor``;
* outputs are freshly allocated on the input's device and fully written;
* inputs must share a device and be contiguous (RadonTorch.cpp:12-14);
  violations raise ``RuntimeError`` like ``AT_ASSERTM`` does;
* batch and channel dimensions are folded together (RadonTorch.cpp:30-37).

Deliberate differences (all in the caller's favour):

* the compute runs in ``libpridediff_dd.so`` on the current CUDA stream;
  CPU tensors raise ``RuntimeError`` (the build has no CPU fallback);
* ``options`` is read on the host once per (tensor, version) and cached, so
  repeated calls do not synchronise with the device (the reference calls
  ``.item()`` 11-17 times per call, RadonTorch.cpp:19-29);
* launch and argument errors are reported (the reference checks none), and
  a device-side wait that timed out in an earlier call makes the next call
  raise (``status.check``; the reference has no device-side waits).
"""
from __future__ import annotations

import torch

from . import _native as N
from . import status as _status

# ---------------------------------------------------------------------------
# options on the host
# ---------------------------------------------------------------------------
_opt_cache: list = []   # (weakref(tensor), version, values) for device-resident options


def host_options(options):
    """Python floats of an options vector without re-reading device memory.

    Host tensors and sequences are read directly.  For a device tensor (the
    reference moves projector.options to the GPU) the values are cached per
    tensor object and version, so repeated calls do not synchronise.
    """
    import weakref
    if isinstance(options, (list, tuple)):
        return [float(x) for x in options]
    if not isinstance(options, torch.Tensor):
        raise RuntimeError("options must be a tensor or a sequence of numbers")
    if options.device.type == "cpu":
        return [float(x) for x in options.detach().double().reshape(-1).tolist()]
    for ref, ver, vals in _opt_cache:
        if ref() is options and ver == options._version:
            return vals
    vals = [float(x) for x in options.detach().to("cpu", torch.float64).reshape(-1).tolist()]
    _opt_cache[:] = [e for e in _opt_cache if e[0]() is not None][-63:]
    _opt_cache.append((weakref.ref(options), options._version, vals))
    return vals


def _check_inputs(x: torch.Tensor, angles: torch.Tensor, extra=None):
    # CHECK_DEVICE / CHECK_CONTIGUOUS (RadonTorch.cpp:12-14)
    tensors = [x, angles] + ([extra] if extra is not None else [])
    dev = x.device
    if any(t.device != dev for t in tensors):
        raise RuntimeError("Expected all tensors to be on the same device")
    if any(not t.is_contiguous() for t in tensors):
        raise RuntimeError("Expected all tensors to be contiguous")
    if dev.type != "cuda":
        raise RuntimeError("pridediff_gb300 runs on CUDA devices only; got a tensor on " + str(dev))
    if x.dtype != torch.float32 or angles.dtype != torch.float32:
        raise RuntimeError("Expected float32 tensors")


def _stream_ptr(dev):
    return torch.cuda.current_stream(dev).cuda_stream


def _plan_budget() -> int:
    import os
    return int(os.environ.get("PRIDEDIFF_PLAN_CACHE_BYTES", str(16 << 30)))


class _PlanCache:
    """Geometry plans keyed by (scan, geometry, angles tensor identity/version).

    A plan holds the per-view detector tables, the per-line drift pieces and,
    for fan beams, the adjoint map (about 1.8 GB for 512^2 pixels and 720
    views); it depends only on the geometry and the angles, so iterative
    callers (the data-consistency loop, autograd forward + backward) build it
    once -- as long as they pass the same angles tensor: the key is the
    tensor's identity and version, never its values (reading them would
    synchronise), so an angles tensor rebuilt every call (a fresh
    torch.arange) rebuilds the plan every call.  The entry keeps a weak
    reference to the angles tensor so a new tensor that happens to reuse the
    same memory is never mistaken for the old one.

    At most `size` plans and `budget` bytes of them are kept (least recently
    used first out; the newest plan is always kept); the byte budget defaults
    to 16 GiB (PRIDEDIFF_PLAN_CACHE_BYTES).  `nbytes()` reports what is held,
    `clear()` releases it.
    """

    def __init__(self, size: int = 8, budget: int = None):
        self.size = size
        self.budget = _plan_budget() if budget is None else budget
        self.entries = []   # (key, weakref(angles), version, plan entry, bytes)

    @staticmethod
    def _bytes(entry) -> int:
        plan = entry[0] if isinstance(entry, tuple) else entry
        return int(plan.numel()) * int(plan.element_size())

    def get(self, key, angles, build):
        import weakref
        for i, (k, ref, ver, plan, _) in enumerate(self.entries):
            if k == key and ref() is angles and ver == angles._version:
                self.entries.insert(0, self.entries.pop(i))
                return plan
        plan = build()
        self.entries.insert(0, (key, weakref.ref(angles), angles._version, plan, self._bytes(plan)))
        del self.entries[self.size:]
        while len(self.entries) > 1 and self.nbytes() > self.budget:
            self.entries.pop()
        return plan

    def nbytes(self) -> int:
        return sum(e[4] for e in self.entries)

    def clear(self):
        self.entries.clear()


plans = _PlanCache()


def plan2d(scan: str, g, angles: torch.Tensor):
    """Device plan of a 2-D geometry (cached)."""
    lib = N.load()
    sc = N.SCAN2D[scan]
    V = int(angles.shape[0])
    key = ("2d", sc, tuple(getattr(g, f) for f, _ in g._fields_), V, angles.device.index)

    def build():
        nbytes = int(lib.dd2d_plan_bytes(sc, g, V))
        plan = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=angles.device)
        N.check(lib.dd2d_plan(sc, g, angles.data_ptr(), V, plan.data_ptr(), nbytes,
                              _stream_ptr(angles.device)), f"{scan} plan")
        return plan

    return plans.get(key, angles, build)


def _apply2d(scan: str, op: str, x: torch.Tensor, options, angles: torch.Tensor) -> torch.Tensor:
    _check_inputs(x, angles)
    lib = N.load()
    o = host_options(options)
    g = N.geom2d(o)
    if x.dim() != 4:
        raise RuntimeError("expected a 4-D (B, C, ., .) tensor")
    B, C = x.shape[0], x.shape[1]
    V = angles.shape[0]
    image_in = op in ("proj", "bproj_t", "bproj_tw")
    if image_in:
        if (x.shape[2], x.shape[3]) != (g.height, g.width):
            raise RuntimeError("image size inconsistent with options")
        out = torch.empty((B, C, V, g.num_det), dtype=torch.float32, device=x.device)
    else:
        if (x.shape[2], x.shape[3]) != (V, g.num_det):
            raise RuntimeError("sinogram size inconsistent with options and angles")
        out = torch.empty((B, C, g.height, g.width), dtype=torch.float32, device=x.device)
    if B * C == 0:
        return out.zero_()
    sc, opc = N.SCAN2D[scan], N.OPS[op]
    _status.check(x.device)
    with torch.cuda.device(x.device):
        # the library validates the geometry before anything is enqueued
        N.check(lib.dd2d_validate(sc, opc, g, B * C, V), f"{scan} {op}")
        plan = plan2d(scan, g, angles)
        nbytes = int(lib.dd2d_apply_workspace_bytes(sc, opc, g, B * C, V))
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)

        def run(cfg):
            return lib.dd2d_apply_planned_tuned(sc, opc, g, plan.data_ptr(), x.data_ptr(), out.data_ptr(), B * C,
                                                V, ws.data_ptr(), nbytes, forward_tune(cfg),
                                                _stream_ptr(x.device))
        cfg = forward_shape(sc, g, B * C, V, x.device, run) if image_in else None
        st = run(cfg)
    N.check(st, f"{scan} {op}")
    return out


def forward_tune(cfg):
    """dd_tune2d for a forward shape {fwd_slices, fwd_cluster} (None: defaults)."""
    t = N.Tune2d()
    if cfg:
        t.fwd_slices = int(cfg.get("fwd_slices", 0))
        t.fwd_cluster = int(cfg.get("fwd_cluster", 0))
    return t


def forward_shape(sc: int, g, batch: int, views: int, device, run):
    """The single-geometry forward's CTA shape for this geometry and batch,
    chosen by the autotuner on first use (timing every candidate on the
    call's own buffers, which the chosen shape then overwrites) and kept for
    the process and in the tuner's cache; the library's defaults while a
    stream is being captured or when tuning is off (PRIDEDIFF_AUTOTUNE=0)."""
    from . import autotune
    if not autotune.enabled():
        return None
    key = autotune.forward2d_key(sc, tuple(getattr(g, f) for f, _ in g._fields_), batch, views, device)
    if key in autotune._forward_choice:
        return autotune._forward_choice[key]
    if torch.cuda.is_current_stream_capturing():
        return None

    def launch(cfg):
        N.check(run(cfg), "forward tuning")
    about = {"scan": {v: k for k, v in N.SCAN2D.items()}[sc], "image": [g.width, g.height], "dets": g.num_det,
             "views": views, "batch": batch}
    return autotune.tune_forward2d(key, launch, about=about)


def plan3d(scan: str, g, angles: torch.Tensor, source_pos=None):
    """Device plan of a 3-D geometry (cached; spiral plans also key on the
    source table's identity and version)."""
    lib = N.load()
    sc = N.SCAN3D[scan]
    V = int(angles.shape[0])
    sp_key = None if source_pos is None else (id(source_pos), source_pos._version)
    key = ("3d", sc, tuple(getattr(g, f) for f, _ in g._fields_), V, angles.device.index, sp_key)

    def build():
        nbytes = int(lib.dd3d_plan_bytes(sc, g, V))
        plan = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=angles.device)
        N.check(lib.dd3d_plan(sc, g, angles.data_ptr(), source_pos.data_ptr() if source_pos is not None else None,
                              V, plan.data_ptr(), nbytes, _stream_ptr(angles.device)), f"{scan} plan")
        # keep the source table alive as long as the plan is cached
        return (plan, source_pos) if source_pos is not None else plan

    entry = plans.get(key, angles, build)
    return entry[0] if isinstance(entry, tuple) else entry


def _apply3d(scan: str, op: str, x: torch.Tensor, options, angles: torch.Tensor, source_pos=None) -> torch.Tensor:
    _check_inputs(x, angles, source_pos)
    if source_pos is not None and source_pos.dtype != torch.float32:
        raise RuntimeError("Expected float32 tensors")
    lib = N.load()
    o = host_options(options)
    g = N.geom3d(o, spiral=(scan == "spiral"))
    if x.dim() != 5:
        raise RuntimeError("expected a 5-D (B, C, ., ., .) tensor")
    B, Ch = x.shape[0], x.shape[1]
    V = angles.shape[0]
    if scan == "spiral" and (source_pos is None or tuple(source_pos.shape) != (4, V)):
        raise RuntimeError("source_pos must be a (4, V) tensor")
    image_in = op in ("proj", "bproj_t", "bproj_tw")
    if image_in:
        if tuple(x.shape[2:]) != (g.depth, g.height, g.width):
            raise RuntimeError("image size inconsistent with options")
        out = torch.empty((B, Ch, V, g.num_row, g.num_col), dtype=torch.float32, device=x.device)
    else:
        if tuple(x.shape[2:]) != (V, g.num_row, g.num_col):
            raise RuntimeError("sinogram size inconsistent with options and angles")
        out = torch.empty((B, Ch, g.depth, g.height, g.width), dtype=torch.float32, device=x.device)
    if B * Ch == 0:
        return out.zero_()
    sc, opc = N.SCAN3D[scan], N.OPS[op]
    _status.check(x.device)
    with torch.cuda.device(x.device):
        N.check(lib.dd3d_validate(sc, opc, g, B * Ch, V), f"{scan} {op}")
        plan = plan3d(scan, g, angles, source_pos)
        nbytes = int(lib.dd3d_apply_workspace_bytes(sc, opc, g, B * Ch, V))
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
        st = lib.dd3d_apply_planned(sc, opc, g, plan.data_ptr(), x.data_ptr(), out.data_ptr(), B * Ch, V,
                                    ws.data_ptr(), nbytes, _stream_ptr(x.device))
    N.check(st, f"{scan} {op}")
    return out


# ---------------------------------------------------------------------------
# 2-D operators (RadonTorch.cpp:1376-1393)
# ---------------------------------------------------------------------------
def _mk2(scan, op, name):
    def f(input, options, angles):
        return _apply2d(scan, op, input, options, angles)
    f.__name__ = name
    f.__doc__ = f"Replaces radontorch.{name} (deeprecon/interface/RadonTorch.cpp)."
    return f


_NAMES2D = {
    "FanFlat": "flat", "FanArc": "arc",
}
for _n, _s in _NAMES2D.items():
    for _pre, _op in (("Proj", "proj"), ("ProjTrans", "proj_t"), ("BackProj", "bproj"),
                      ("BackProjTrans", "bproj_t"), ("BackProjWeighted", "bproj_w"),
                      ("BackProjTransWeighted", "bproj_tw")):
        _name = f"{_pre}{_n}Dis2d"
        globals()[_name] = _mk2(_s, _op, _name)
for _pre, _op in (("Proj", "proj"), ("ProjTrans", "proj_t"), ("BackProj", "bproj"),
                  ("BackProjTrans", "bproj_t")):
    _name = f"{_pre}ParaDis2d"
    globals()[_name] = _mk2("para", _op, _name)

# ---------------------------------------------------------------------------
# 3-D operators (RadonTorch.cpp:1395-1414)
# ---------------------------------------------------------------------------
def _mk3(scan, op, name):
    if scan == "spiral":
        def f(input, options, angles, source_pos):
            return _apply3d(scan, op, input, options, angles, source_pos)
    else:
        def f(input, options, angles):
            return _apply3d(scan, op, input, options, angles)
    f.__name__ = name
    f.__doc__ = f"Replaces radontorch.{name} (deeprecon/interface/RadonTorch.cpp)."
    return f


NAMES3D = []
for _geo, _s in (("ConeFlat", "cone_flat"), ("ConeArc", "cone_arc"), ("Spiral", "spiral")):
    for _pre, _op in (("Proj", "proj"), ("ProjTrans", "proj_t"), ("BackProj", "bproj"),
                      ("BackProjTrans", "bproj_t"), ("BackProjWeighted", "bproj_w"),
                      ("BackProjTransWeighted", "bproj_tw")):
        _name = f"{_pre}{_geo}Dis3d"
        globals()[_name] = _mk3(_s, _op, _name)
        NAMES3D.append(_name)

# ---------------------------------------------------------------------------
# System matrices (RadonTorch.cpp:1270-1372)
# ---------------------------------------------------------------------------
def _sysmatrix(scan: str, options, angles: torch.Tensor) -> torch.Tensor:
    """COO system matrix (V*D x H*W) of a 2-D geometry, built on the GPU.

    Same entries, order and CPU sparse result as deeprecon's builders (one
    entry per step of the DD merge walk, view by view and line by line).  The
    reference accepts CPU tensors only (its Python wrapper moves them there,
    function.py:535-553); here CPU and CUDA inputs are both accepted and the
    work runs on the current CUDA device.
    """
    if not torch.cuda.is_available():
        raise RuntimeError("pridediff_gb300 builds the system matrix on a CUDA device; none is available")
    lib = N.load()
    g = N.geom2d(host_options(options))
    dev = angles.device if angles.device.type == "cuda" else torch.device("cuda", torch.cuda.current_device())
    ang = angles.detach().to(dev, torch.float32).contiguous()
    V = int(ang.shape[0])
    sc = N.SCAN2D[scan]
    _status.check(dev)
    with torch.cuda.device(dev):
        N.check(lib.dd2d_validate(sc, N.OPS["proj"], g, 1, V), f"{scan} system matrix")
        plan = plan2d(scan, g, ang)
        n_lines = int(lib.dd2d_sysmatrix_lines(g, V))
        counts = torch.empty(n_lines, dtype=torch.int64, device=dev)
        N.check(lib.dd2d_sysmatrix_count(sc, g, plan.data_ptr(), V, counts.data_ptr(), _stream_ptr(dev)),
                f"{scan} system matrix")
        offsets = torch.cumsum(counts, 0) - counts
        nnz = int(counts.sum().item())
        rows = torch.empty(max(nnz, 1), dtype=torch.int64, device=dev)
        cols = torch.empty(max(nnz, 1), dtype=torch.int64, device=dev)
        vals = torch.empty(max(nnz, 1), dtype=torch.float32, device=dev)
        N.check(lib.dd2d_sysmatrix_fill(sc, g, plan.data_ptr(), V, offsets.data_ptr(), rows.data_ptr(),
                                        cols.data_ptr(), vals.data_ptr(), _stream_ptr(dev)), f"{scan} system matrix")
    indices = torch.stack([rows[:nnz], cols[:nnz]]).cpu()
    return torch.sparse_coo_tensor(indices, vals[:nnz].cpu(), (V * g.num_det, g.height * g.width),
                                   dtype=torch.float32)


def GetSysMatrixFanFlat2d(options, angles):
    """Replaces radontorch.GetSysMatrixFanFlat2d (deeprecon/interface/RadonTorch.cpp:1270)."""
    return _sysmatrix("flat", options, angles)


def GetSysMatrixFanArc2d(options, angles):
    """Replaces radontorch.GetSysMatrixFanArc2d (deeprecon/interface/RadonTorch.cpp:1305)."""
    return _sysmatrix("arc", options, angles)


def GetSysMatrixPara2d(options, angles):
    """Replaces radontorch.GetSysMatrixPara2d (deeprecon/interface/RadonTorch.cpp:1340)."""
    return _sysmatrix("para", options, angles)

NAMES2D = [n for n in globals() if n.endswith("Dis2d")]
ALL_NAMES = NAMES2D + NAMES3D + ["GetSysMatrixFanFlat2d", "GetSysMatrixFanArc2d", "GetSysMatrixPara2d"]

"""Uneven batches of 2-D projections in one persistent launch, and the
graph-captured data-consistency (DC) loop.

``UnevenBatch2d`` takes a list of ``projector2d`` modules of one scan type
(each with its own image size, detector count and angles) and runs the
forward projection, the exact adjoint, or the DC step
``x <- x - eta * A^T (A x - y)`` of all of them together: one persistent
kernel launch per operator, work items pulled longest-first from a device
counter (``libpridediff_dd.so``: dd2d_batch_*).

Tensors are packed into flat float32 tensors; ``pack`` and ``unpack_*``
convert from/to lists of (batch_i, 1, H_i, W_i) images or (batch_i, 1, V_i,
D_i) sinograms, one per instance in the order given.  Instances with the same
geometry and the same view angles are merged into one multi-slice instance
(``group=True``, the default): their slices then share each work item's
per-line set-up and each adjoint-map block read, and the packed layout keeps
a group's slices together (``pack`` / ``unpack_*`` apply that order).  Merging
changes no arithmetic: every slice's result is the same bit for bit.

``dc_graph`` captures ``steps`` DC steps in one CUDA graph: replaying it
launches no host work at all.  The reference runs each step as separate
operator calls with host syncs and per-call allocations
(model/pridediff.py:56-68, RadonTorch.cpp:19-33).
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import torch

from . import _native as N
from . import status as _status
from .radontorch import host_options


class UnevenBatch2d:
    def __init__(self, projectors: Sequence, angles: Sequence[torch.Tensor],
                 batch: Optional[Sequence[int]] = None, tune: Optional[dict] = None, group: bool = True):
        if len(projectors) == 0 or len(projectors) != len(angles):
            raise ValueError("need one angles tensor per projector")
        scans = {p.scan_type for p in projectors}
        if len(scans) != 1:
            raise ValueError("an uneven batch holds one scan type")
        self.scan = scans.pop()
        self.sc = N.SCAN2D[self.scan]
        self.device = angles[0].device
        if self.device.type != "cuda":
            raise RuntimeError("UnevenBatch2d runs on CUDA devices only")
        self.angles = [a.contiguous() for a in angles]
        if any(a.device != self.device or a.dtype != torch.float32 for a in self.angles):
            raise RuntimeError("angles must be float32 tensors on one CUDA device")
        self.batch = list(batch) if batch is not None else [1] * len(projectors)
        self.geoms = [N.geom2d(host_options(p.options)) for p in projectors]
        self.img_shapes = [(b, 1, g.height, g.width) for g, b in zip(self.geoms, self.batch)]
        self.sino_shapes = [(b, 1, int(a.shape[0]), g.num_det) for g, a, b in zip(self.geoms, self.angles, self.batch)]
        self.img_numel = sum(s[0] * s[2] * s[3] for s in self.img_shapes)
        self.sino_numel = sum(s[0] * s[2] * s[3] for s in self.sino_shapes)
        # groups of instances with the same geometry and angles, in order of first appearance
        self.groups: List[List[int]] = []
        keys = []
        for i, (g, a) in enumerate(zip(self.geoms, self.angles)):
            key = tuple(getattr(g, f) for f, _ in g._fields_) + (int(a.shape[0]),)
            for gi, k in enumerate(keys):
                if group and k == key and torch.equal(self.angles[self.groups[gi][0]], a):
                    self.groups[gi].append(i)
                    break
            else:
                keys.append(key)
                self.groups.append([i])
        n = len(self.groups)
        self.n = n
        self.inst = (N.Instance2d * n)()
        for gi, members in enumerate(self.groups):
            i0 = members[0]
            self.inst[gi].geom = self.geoms[i0]
            self.inst[gi].num_view = int(self.angles[i0].shape[0])
            self.inst[gi].batch = sum(int(self.batch[i]) for i in members)
        self._order = [i for members in self.groups for i in members]   # packed order of the instances
        self._img_off = self._offsets(self.img_shapes)
        self._sino_off = self._offsets(self.sino_shapes)
        self.tune = N.Tune2d()
        self.set_tune(tune or {})
        self._plan()

    # -- configuration -------------------------------------------------------
    def set_tune(self, tune: dict):
        self.tune.ctas_per_sm = int(tune.get("ctas_per_sm", 0))
        self.tune.lpt_order = int(tune.get("lpt_order", 1))
        self.tune.items_cluster = int(tune.get("items_cluster", 1))
        self.tune_dict = {"ctas_per_sm": self.tune.ctas_per_sm, "lpt_order": self.tune.lpt_order,
                          "items_cluster": self.tune.items_cluster}
        if hasattr(self, "plan"):
            self._plan()

    def _plan(self):
        lib = N.load()
        nb = int(lib.dd2d_batch_plan_bytes(self.sc, self.inst, self.n))
        if nb == 0:
            N.check(lib.dd2d_validate(self.sc, N.OPS["proj"], ctypes.byref(self.geoms[0]), 1, 1) or
                    N.DD_ERR_INVALID_ARG, "uneven batch")
        self.plan = torch.empty(nb, dtype=torch.uint8, device=self.device)
        ptrs = (ctypes.c_void_p * self.n)(*[self.angles[m[0]].data_ptr() for m in self.groups])
        with torch.cuda.device(self.device):
            N.check(lib.dd2d_batch_plan(self.sc, self.inst, self.n, ptrs, self.plan.data_ptr(), nb,
                                        ctypes.byref(self.tune), self._stream()), "uneven batch plan")
        wb = int(lib.dd2d_batch_workspace_bytes(self.sc, self.inst, self.n))
        self.workspace = torch.empty(wb, dtype=torch.uint8, device=self.device)

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    # -- packing ---------------------------------------------------------------
    def _offsets(self, shapes):
        """Offset of each instance's block in the packed order."""
        off, o = [0] * len(shapes), 0
        for i in self._order:
            off[i] = o
            o += shapes[i][0] * shapes[i][2] * shapes[i][3]
        return off

    def pack(self, xs: List[torch.Tensor]) -> torch.Tensor:
        """One flat tensor from per-instance images (or sinograms), in the packed order."""
        return torch.cat([xs[i].reshape(-1) for i in self._order]).contiguous()

    def _unpack(self, flat, shapes, off):
        return [flat[o:o + s[0] * s[2] * s[3]].view(s) for s, o in zip(shapes, off)]

    def unpack_images(self, flat: torch.Tensor) -> List[torch.Tensor]:
        return self._unpack(flat, self.img_shapes, self._img_off)

    def unpack_sinos(self, flat: torch.Tensor) -> List[torch.Tensor]:
        return self._unpack(flat, self.sino_shapes, self._sino_off)

    # -- operators -------------------------------------------------------------
    def _apply(self, op: str, x: torch.Tensor) -> torch.Tensor:
        lib = N.load()
        fwd = op in ("proj", "bproj_t")
        if x.numel() != (self.img_numel if fwd else self.sino_numel) or not x.is_contiguous():
            raise RuntimeError("packed input has the wrong size or is not contiguous")
        out = torch.empty(self.sino_numel if fwd else self.img_numel, dtype=torch.float32, device=self.device)
        _status.check(self.device)
        with torch.cuda.device(self.device):
            st = lib.dd2d_batch_apply(self.sc, N.OPS[op], self.inst, self.n, self.plan.data_ptr(), x.data_ptr(),
                                      out.data_ptr(), self.workspace.data_ptr(), self.workspace.numel(),
                                      ctypes.byref(self.tune), self._stream())
        N.check(st, f"uneven batch {op}")
        return out

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        """A x for all instances (packed)."""
        return self._apply("proj", x)

    def adjoint(self, y: torch.Tensor) -> torch.Tensor:
        """A^T y for all instances (packed), the exact adjoint of forward."""
        return self._apply("proj_t", y)

    def project(self, x: torch.Tensor) -> torch.Tensor:
        """Differentiable A x (backward: exact adjoint)."""
        return _BatchProject.apply(x, self)

    def dc_step(self, x: torch.Tensor, y: torch.Tensor, eta: float) -> torch.Tensor:
        """In place: x <- x - eta * A^T (A x - y)."""
        lib = N.load()
        if x.numel() != self.img_numel or y.numel() != self.sino_numel:
            raise RuntimeError("packed x / y have the wrong size")
        _status.check(self.device)
        with torch.cuda.device(self.device):
            st = lib.dd2d_batch_dc_step(self.sc, self.inst, self.n, self.plan.data_ptr(), x.data_ptr(),
                                        y.data_ptr(), float(eta), self.workspace.data_ptr(),
                                        self.workspace.numel(), ctypes.byref(self.tune), self._stream())
        N.check(st, "uneven batch dc step")
        return x

    def device_status(self) -> int:
        s = ctypes.c_int(-1)
        N.check(N.load().dd2d_batch_status(self.sc, self.inst, self.n, self.workspace.data_ptr(), ctypes.byref(s)),
                "status")
        return s.value

    def dc_graph(self, x: torch.Tensor, y: torch.Tensor, eta: float, steps: int):
        """Capture `steps` DC steps on (x, y) in one CUDA graph; returns it.

        Replay with ``g.replay()``; x is updated in place.  x and y must stay
        alive (the graph holds their addresses)."""
        self.dc_step(x.clone(), y, 0.0)   # warm-up outside capture (kernel attributes)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(steps):
                    self.dc_step(x, y, eta)
        torch.cuda.current_stream(self.device).wait_stream(s)
        return g


class _BatchProject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, batch):
        ctx.batch = batch
        return batch.forward(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        return ctx.batch.adjoint(g.contiguous()), None

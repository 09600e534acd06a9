"""The timeout path of the bounded device-side waits, run on a GPU.

The library's kernels wait on asynchronous bulk copies with a bounded number
of polls.  This test loads a separate build of the library in which every
such wait gives up at once (DD_WAIT_LIMIT=0; _native.VARIANTS) and calls each
kernel family through the C ABI: the fan- and parallel-beam single-geometry
forward and adjoints, the persistent uneven-batch forward and adjoint, the
3-D forward and adjoint and the no-allocation entry point.  Each call must
return (its kernels skip their work, let the copies they issued land and
record DD_ERR_TIMEOUT), its status reader must report DD_ERR_TIMEOUT, the
pinned host word registered with dd_set_status_sink must show it without a
synchronisation, and the CUDA context must stay usable: the product library
still computes correct results afterwards.  No wait is left to spin and no
kernel faults: the drain after a timeout keeps its own, full-length bound.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def waitlib():
    from pridediff_gb300 import _native as N
    lib = N.load_variant("waittest")
    word = torch.zeros(1, dtype=torch.int32, pin_memory=True)
    assert lib.dd_set_status_sink(word.data_ptr()) == N.DD_OK
    yield N, lib, word
    torch.cuda.synchronize()
    assert lib.dd_set_status_sink(None) == N.DD_OK


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _expect_timeout(N, word, read):
    torch.cuda.synchronize()          # the calls returned and their kernels ended
    s = ctypes.c_int(-1)
    assert read(ctypes.byref(s)) == N.DD_OK
    assert s.value == N.DD_ERR_TIMEOUT, N.status_string(s.value)
    assert int(word[0]) == N.DD_ERR_TIMEOUT
    word[0] = 0


@pytest.mark.parametrize("scan,op", [("flat", "proj"), ("flat", "proj_t"), ("arc", "bproj_w"),
                                     ("para", "proj"), ("para", "proj_t"), ("flat", "bproj_tw")])
def test_2d_single_geometry_timeouts(waitlib, scan, op):
    N, lib, word = waitlib
    D = 80
    g = N.Geom2d(64, 48, D, 1.0, 1.0, 1.3 if scan != "arc" else 1.3 / 1000.0, 500.0, 1000.0, 0.0, 0.0, 0.0)
    V, B = 24, 2
    ang = torch.arange(V, dtype=torch.float32, device="cuda") * (2 * np.pi / V)
    image_in = op in ("proj", "bproj_t", "bproj_tw")
    x = torch.rand((B, 48, 64) if image_in else (B, V, D), device="cuda")
    out = torch.zeros((B, V, D) if image_in else (B, 48, 64), device="cuda")
    sc, opc = N.SCAN2D[scan], N.OPS[op]
    nbytes = lib.dd2d_workspace_bytes(sc, opc, ctypes.byref(g), B, V)
    ws = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    st = lib.dd2d_apply(sc, opc, ctypes.byref(g), x.data_ptr(), out.data_ptr(), ang.data_ptr(), B, V,
                        ws.data_ptr(), nbytes, _stream())
    assert st == N.DD_OK
    _expect_timeout(N, word, lambda p: lib.dd2d_status(sc, opc, ctypes.byref(g), B, V, ws.data_ptr(), p))


def test_uneven_batch_timeouts(waitlib):
    N, lib, word = waitlib
    sizes = [(64, 24, 80), (48, 16, 72), (96, 20, 100)]
    inst = (N.Instance2d * len(sizes))()
    angs = []
    for i, (n, V, D) in enumerate(sizes):
        inst[i].geom = N.Geom2d(n, n, D, 1.0, 1.0, 1.3, 500.0, 1000.0, 0.0, 0.0, 0.0)
        inst[i].num_view = V
        inst[i].batch = 1
        angs.append(torch.arange(V, dtype=torch.float32, device="cuda") * (2 * np.pi / V))
    sc = N.SCAN2D["flat"]
    tune = N.Tune2d(0, 1)
    pb = lib.dd2d_batch_plan_bytes(sc, inst, len(sizes))
    plan = torch.zeros(pb, dtype=torch.uint8, device="cuda")
    ptrs = (ctypes.c_void_p * len(sizes))(*[a.data_ptr() for a in angs])
    assert lib.dd2d_batch_plan(sc, inst, len(sizes), ptrs, plan.data_ptr(), pb, ctypes.byref(tune), _stream()) == 0
    wb = lib.dd2d_batch_workspace_bytes(sc, inst, len(sizes))
    ws = torch.zeros(wb, dtype=torch.uint8, device="cuda")
    n_img = sum(n * n for n, _, _ in sizes)
    n_sino = sum(V * D for _, V, D in sizes)
    for op, nin, nout in (("proj", n_img, n_sino), ("proj_t", n_sino, n_img)):
        x = torch.rand(nin, device="cuda")
        out = torch.zeros(nout, device="cuda")
        st = lib.dd2d_batch_apply(sc, N.OPS[op], inst, len(sizes), plan.data_ptr(), x.data_ptr(), out.data_ptr(),
                                  ws.data_ptr(), wb, ctypes.byref(tune), _stream())
        assert st == N.DD_OK
        _expect_timeout(N, word, lambda p: lib.dd2d_batch_status(sc, inst, len(sizes), ws.data_ptr(), p))


@pytest.mark.parametrize("scan,op", [("cone_flat", "proj"), ("cone_flat", "proj_t"), ("spiral", "proj"),
                                     ("spiral", "bproj")])
def test_3d_timeouts(waitlib, scan, op):
    import cases3d
    N, lib, word = waitlib
    name = "cone_flat_small" if scan == "cone_flat" else "spiral_small"
    geom, opt, ang_np, sp_np = cases3d.cases()[name]
    g = N.geom3d([float(v) for v in opt], spiral=(scan == "spiral"))
    V, B = len(ang_np), 2
    x_np, y_np = cases3d.inputs(cases3d.cases()[name], batch=B, seed=3)
    x = torch.from_numpy(x_np if op == "proj" else y_np).cuda()
    out = torch.zeros(tuple((y_np if op == "proj" else x_np).shape), device="cuda")
    ang = torch.from_numpy(ang_np).cuda()
    sp = torch.from_numpy(sp_np).cuda() if sp_np is not None else None
    sc, opc = N.SCAN3D[scan], N.OPS[op]
    nbytes = lib.dd3d_workspace_bytes(sc, opc, ctypes.byref(g), B, V)
    ws = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    st = lib.dd3d_apply(sc, opc, ctypes.byref(g), x.data_ptr(), out.data_ptr(), ang.data_ptr(),
                        sp.data_ptr() if sp is not None else None, B, V, ws.data_ptr(), nbytes, _stream())
    assert st == N.DD_OK
    _expect_timeout(N, word, lambda p: lib.dd3d_status(sc, opc, ctypes.byref(g), B, V, ws.data_ptr(), p))


def test_noalloc_timeout(waitlib):
    N, lib, word = waitlib
    lib.dd_ProjFanFlatDis2d_noalloc.restype = ctypes.c_int
    lib.dd_ProjFanFlatDis2d_noalloc.argtypes = [ctypes.POINTER(N.Geom2d)] + [ctypes.c_void_p] * 3 + \
        [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    g = N.Geom2d(64, 64, 92, 2.0, 2.0, 2.6, 595.0, 1085.6, 0.0, 0.0, 0.0)
    V, B = 30, 1
    ang = torch.arange(V, dtype=torch.float32, device="cuda") * (2 * np.pi / V)
    x = torch.rand((B, 64, 64), device="cuda")
    out = torch.zeros((B, V, 92), device="cuda")
    st = lib.dd_ProjFanFlatDis2d_noalloc(ctypes.byref(g), x.data_ptr(), out.data_ptr(), ang.data_ptr(), B, V,
                                         _stream())
    assert st == N.DD_OK
    _expect_timeout(N, word, lambda p: lib.dd_noalloc_status(p))


def test_context_survives_and_product_path_is_correct(waitlib, oracle_mod):
    """After every kernel family timed out, the product library still runs and
    agrees with the oracle, and its own status word stays clear."""
    import pridediff_gb300 as P
    proj = P.projector2d(64, 80, 1.0, 1.3, 500.0, 1000.0, scan_type="flat").cuda()
    ang_np = (np.arange(24) * 2 * np.pi / 24).astype(np.float32)
    x_np = np.random.default_rng(4).random((2, 1, 64, 64)).astype(np.float32)
    y = proj.projection(torch.from_numpy(x_np).cuda(), torch.from_numpy(ang_np).cuda())
    torch.cuda.synchronize()
    ref = oracle_mod.run2d("flat", "proj", x_np[:, 0], ang_np, proj.options.cpu().numpy(), "f", 0)
    assert rel_l2(y[:, 0].cpu().numpy(), ref) <= 1e-5
    assert P.device_status() == 0


def test_product_reports_a_recorded_timeout_on_the_next_call():
    """A timeout recorded in the product's host word (as a kernel would write
    it) makes the next operator call raise, without any synchronisation."""
    import pridediff_gb300 as P
    from pridediff_gb300 import status
    proj = P.projector2d(32, 40, 1.0, 1.3, 500.0, 1000.0, scan_type="flat").cuda()
    ang = torch.arange(8, dtype=torch.float32, device="cuda")
    x = torch.rand((1, 1, 32, 32), device="cuda")
    proj.projection(x, ang)                        # registers the device
    status._word[0] = 5                            # DD_ERR_TIMEOUT, as dd_report_timeout writes it
    with pytest.raises(RuntimeError, match="timed out"):
        proj.projection(x, ang)
    assert int(status._word[0]) == 0               # reported once, then cleared
    proj.projection(x, ang)

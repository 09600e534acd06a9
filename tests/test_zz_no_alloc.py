"""The fan-flat forward projection that allocates nothing.

Some callers cannot call cudaMalloc at all: a plugin whose host framework
owns all device memory, or a real-time loop that may not touch the
allocator.  dd_ProjFanFlatDis2d_noalloc serves them from a fixed 32 MiB
buffer inside the library.  This test calls it through the C ABI, twice in a
row with different inputs, and checks each result against the regular entry
point dd_ProjFanFlatDis2d (which takes caller-provided workspace): the same
kernels on the same inputs, so the results must be bit-equal.  The file
name sorts last so that a run stopping at its first failure has run every
other test first; it also passes when run alone.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lib():
    from pridediff_gb300 import _native as N
    lib = N.load()
    g2 = ctypes.POINTER(N.Geom2d)
    vp, i = ctypes.c_void_p, ctypes.c_int
    lib.dd_ProjFanFlatDis2d_noalloc.restype = i
    lib.dd_ProjFanFlatDis2d_noalloc.argtypes = [g2, vp, vp, vp, i, i, vp]
    lib.dd_ProjFanFlatDis2d.restype = i
    lib.dd_ProjFanFlatDis2d.argtypes = [g2, vp, vp, vp, i, i, vp, ctypes.c_size_t, vp]
    return N, lib


def test_noalloc_forward_matches_regular_entry_twice():
    N, lib = _lib()
    g = N.Geom2d(128, 128, 184, 2.64, 2.64, 5.1432, 595.0, 1085.6, 0.0, 0.0, 0.0)
    V, B = 180, 2
    ang = torch.arange(V, dtype=torch.float32, device="cuda") * (2 * np.pi / V)
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device="cuda").manual_seed(17)
    for call in range(2):   # two calls in a row share the library's buffer
        x = torch.rand((B, 128, 128), device="cuda", generator=gen) * (call + 1)
        out = torch.empty((B, V, 184), device="cuda")
        ref = torch.empty_like(out)
        st = lib.dd_ProjFanFlatDis2d_noalloc(ctypes.byref(g), x.data_ptr(), out.data_ptr(), ang.data_ptr(),
                                             B, V, stream)
        assert st == N.DD_OK, N.status_string(st)
        nbytes = lib.dd2d_workspace_bytes(1, 0, ctypes.byref(g), B, V)
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        st = lib.dd_ProjFanFlatDis2d(ctypes.byref(g), x.data_ptr(), ref.data_ptr(), ang.data_ptr(), B, V,
                                     ws.data_ptr(), nbytes, stream)
        assert st == N.DD_OK, N.status_string(st)
        torch.cuda.synchronize()
        # the same kernels in the same order on the same inputs: bit-equal
        assert torch.equal(out, ref)
        s = ctypes.c_int(-1)
        assert lib.dd_noalloc_status(ctypes.byref(s)) == N.DD_OK and s.value == N.DD_OK


def test_noalloc_refuses_problems_larger_than_its_buffer():
    N, lib = _lib()
    g = N.Geom2d(512, 512, 736, 0.66, 0.66, 1.2858, 595.0, 1085.6, 0.0, 0.0, 0.0)
    V = 720
    ang = torch.zeros(V, device="cuda")
    x = torch.zeros((1, 512, 512), device="cuda")
    out = torch.zeros((1, V, 736), device="cuda")
    st = lib.dd_ProjFanFlatDis2d_noalloc(ctypes.byref(g), x.data_ptr(), out.data_ptr(), ang.data_ptr(), 1, V,
                                         torch.cuda.current_stream().cuda_stream)
    assert st == N.DD_ERR_WORKSPACE

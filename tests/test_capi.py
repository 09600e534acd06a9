"""The C ABI library: it builds for sm_103a, loads, exports every symbol that
include/pridediff_dd.h declares, and rejects bad arguments with status codes
before touching the device (so these tests need no GPU)."""
import ctypes
import math
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "pridediff_dd.h")


@pytest.fixture(scope="module")
def lib():
    from pridediff_gb300 import _native
    _native.build()
    return _native.load()


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b((?:dd2d|dd3d|dd)_\w+)\s*\(", text))
    # the named-entry macro expands to dd_<name>
    names |= {"dd_" + n for n in re.findall(r"DD_NAMED\dD\((\w+)\);", text)}
    names -= {"dd_" + "##name"}
    return sorted(n for n in names if "##" not in n)


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, f"missing exports: {missing}"


def test_version_and_status_strings(lib):
    assert b"sm_103a" in lib.dd_version()
    for code in range(7):
        assert lib.dd_status_string(code)


def _g(**kw):
    from pridediff_gb300 import _native
    base = dict(width=64, height=64, num_det=90, pix_x=1.0, pix_y=1.0, det_size=1.0, iso_source=500.0,
                source_detector=1000.0, pix_xshift=0.0, pix_yshift=0.0, bin_shift=0.0)
    base.update(kw)
    return _native.Geom2d(**base)


def test_validation_without_device(lib):
    from pridediff_gb300 import _native as N
    ok = _g()
    assert lib.dd2d_validate(1, 0, ok, 4, 180) == N.DD_OK
    assert lib.dd2d_validate(1, 0, None, 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(1, 0, _g(width=0), 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(1, 0, _g(pix_x=math.nan), 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(1, 0, _g(det_size=math.inf), 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(1, 0, _g(det_size=-1.0), 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(1, 0, _g(iso_source=0.0), 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(0, 0, _g(iso_source=0.0), 4, 180) == N.DD_OK   # parallel beam ignores it
    assert lib.dd2d_validate(1, 0, ok, 0, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(1, 0, ok, 4, -1) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(1, 9, ok, 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(7, 0, ok, 4, 180) == N.DD_ERR_INVALID_ARG
    assert lib.dd2d_validate(0, 4, ok, 4, 180) == N.DD_ERR_UNSUPPORTED     # para has no weighted BP
    assert lib.dd2d_validate(1, 0, _g(width=5000), 1, 180) == N.DD_ERR_SIZE_OVERFLOW
    assert lib.dd2d_validate(1, 0, _g(width=4096, height=4096), 200, 180) == N.DD_ERR_SIZE_OVERFLOW
    assert lib.dd2d_validate(1, 0, _g(num_det=100000), 1, 180) == N.DD_ERR_SIZE_OVERFLOW


def test_apply_rejects_missing_workspace_and_pointers(lib):
    from pridediff_gb300 import _native as N
    g = _g()
    # null device pointers and an absent workspace are refused before any launch
    assert lib.dd2d_apply(1, 0, g, None, None, None, 1, 10, None, 0, None) == N.DD_ERR_INVALID_ARG
    fake = ctypes.c_void_p(0x1000)
    assert lib.dd2d_apply(1, 0, g, fake, fake, fake, 1, 10, None, 0, None) == N.DD_ERR_WORKSPACE
    assert lib.dd2d_apply(1, 0, g, fake, fake, fake, 1, 10, fake, 16, None) == N.DD_ERR_WORKSPACE
    # a one-shot adjoint carries the full plan (with the adjoint map); a
    # one-shot forward leaves the map out and needs less than a reusable plan
    need_adj = lib.dd2d_workspace_bytes(1, 1, g, 1, 10)
    assert need_adj > lib.dd2d_plan_bytes(1, g, 10) > 0
    need_fwd = lib.dd2d_workspace_bytes(1, 0, g, 1, 10)
    assert 0 < need_fwd < need_adj
    assert lib.dd2d_apply(1, 0, g, fake, fake, fake, 1, 10, fake, need_fwd - 1, None) == N.DD_ERR_WORKSPACE
    assert lib.dd2d_plan(1, g, None, 10, fake, 1 << 30, None) == N.DD_ERR_INVALID_ARG


def test_workspace_sizes_scale_with_problem(lib):
    g = _g()
    a = lib.dd2d_apply_workspace_bytes(1, 0, g, 1, 90)
    b = lib.dd2d_apply_workspace_bytes(1, 0, g, 8, 90)
    assert b > a > 0
    assert lib.dd2d_plan_bytes(1, g, 180) > lib.dd2d_plan_bytes(1, g, 90)


def _g3(**kw):
    from pridediff_gb300 import _native
    base = dict(width=64, height=64, depth=32, num_col=128, num_row=64, pix_x=1.0, pix_y=1.0, pix_z=1.0,
                col_size=1.0, row_size=1.0, iso_source=500.0, source_detector=1000.0, pix_xshift=0.0,
                pix_yshift=0.0, pix_zshift=0.0, col_shift=0.0, row_shift=0.0)
    base.update(kw)
    return _native.Geom3d(**base)


def test_validation_3d_without_device(lib):
    from pridediff_gb300 import _native as N
    ok = _g3()
    for scan in range(3):
        for op in range(6):
            assert lib.dd3d_validate(scan, op, ok, 2, 90) == N.DD_OK
    assert lib.dd3d_validate(0, 0, None, 2, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(3, 0, ok, 2, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(0, 6, ok, 2, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(0, 0, _g3(depth=0), 2, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(0, 0, _g3(pix_z=-1.0), 2, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(0, 0, _g3(row_size=math.nan), 2, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(0, 0, _g3(col_shift=math.inf), 2, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(0, 0, ok, 0, 90) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_validate(0, 0, _g3(width=2048, height=2048, depth=1024), 1, 90) == N.DD_ERR_SIZE_OVERFLOW
    assert lib.dd3d_validate(0, 0, ok, 1, 70000) == N.DD_ERR_SIZE_OVERFLOW


def test_apply_3d_rejects_missing_workspace_and_pointers(lib):
    from pridediff_gb300 import _native as N
    g = _g3()
    fake = ctypes.c_void_p(0x1000)
    # spiral needs its source table; every entry needs a workspace
    assert lib.dd3d_apply(2, 0, g, fake, fake, fake, None, 1, 10, fake, 1 << 40, None) == N.DD_ERR_INVALID_ARG
    assert lib.dd3d_apply(0, 0, g, fake, fake, fake, None, 1, 10, None, 0, None) == N.DD_ERR_WORKSPACE
    assert lib.dd3d_apply(0, 0, g, None, fake, fake, None, 1, 10, fake, 1 << 40, None) == N.DD_ERR_INVALID_ARG
    need = lib.dd3d_workspace_bytes(0, 0, g, 1, 10)
    assert need > lib.dd3d_plan_bytes(0, g, 10) > 0
    assert lib.dd3d_apply(0, 0, g, fake, fake, fake, None, 1, 10, fake, need - 1, None) == N.DD_ERR_WORKSPACE

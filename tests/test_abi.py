"""The C-ABI library builds, loads and exports every symbol of include/*.h; argument checks
that fail before any device work return their status codes (no GPU needed)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(fk_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from cardiax_gb300 import _native as N
    N.lib()
    lib = ctypes.CDLL(N.lib_path())
    declared = _declared()
    assert len(declared) >= 7
    for name in declared:
        assert hasattr(lib, name), name
    assert set(N.exported_symbols()) <= set(declared)


def test_status_strings():
    from cardiax_gb300 import _native as N
    L = N.lib()
    for code in range(0, 9):
        assert L.fk_status_string(code)
    assert L.fk_status_string(2).decode().startswith("invalid grid")


@pytest.mark.parametrize("H,W,pitch,expect", [(2, 8, 8, 2), (8, 2, 8, 2), (8, 8, 6, 2),
                                              (8, 6, 6, 3)])
def test_shape_checks(H, W, pitch, expect):
    from cardiax_gb300 import _native as N
    L = N.lib()
    p = N.Params(*[1.0] * 14)
    s = (N.Stimulus * 1)()
    ck = (ctypes.c_int64 * 2)(0, 1)
    rc = L.fk_forward(N.Grid(H, W, pitch), 16, 32, 48, ctypes.byref(p), s, 0, ck, 2, 0.01, 0.01,
                      64, None)
    assert rc == expect


def test_null_and_argument_checks():
    from cardiax_gb300 import _native as N
    L = N.lib()
    p = N.Params(*[1.0] * 14)
    s = (N.Stimulus * 9)()
    g = N.Grid(8, 8, 8)
    assert L.fk_forward_euler(g, None, 32, 48, ctypes.byref(p), s, 0, 0, 1, 0.01, 0.01, None) == 1
    assert L.fk_forward_euler(g, 16, 32, 48, ctypes.byref(p), s, 0, 0, 1, 0.01, -1.0, None) == 5
    assert L.fk_forward_euler(g, 16, 32, 48, ctypes.byref(p), s, 0, 5, 1, 0.01, 0.01, None) == 5
    assert L.fk_forward_euler(g, 18, 32, 48, ctypes.byref(p), s, 0, 0, 1, 0.01, 0.01, None) == 3
    assert L.fk_forward_euler(g, 16, 32, 48, ctypes.byref(p), s, 9, 0, 1, 0.01, 0.01, None) == 4
    ck = (ctypes.c_int64 * 3)(0, 5, 3)
    assert L.fk_forward(g, 16, 32, 48, ctypes.byref(p), s, 0, ck, 3, 0.01, 0.01, 64, None) == 5


def test_scar_entry_points_check_arguments():
    """fk_scar_raster / fk_conv2d_same reject bad arguments before any device work."""
    from cardiax_gb300 import _native as N
    L = N.lib()
    off = (ctypes.c_int32 * 3)(0, 5, 10)
    fake = 0x1000  # never dereferenced: each call below fails its host-side checks first
    assert L.fk_scar_raster(fake, fake, off, 2, 16, 16, None, 16, fake, None) == 1
    assert L.fk_scar_raster(fake, fake, None, 2, 16, 16, fake, 16, fake, None) == 1
    assert L.fk_scar_raster(fake, fake, off, 17, 16, 16, fake, 16, fake, None) == 2
    assert L.fk_scar_raster(fake, fake, off, 2, 16, 16, fake, 8, fake, None) == 2
    bad0 = (ctypes.c_int32 * 2)(1, 5)
    assert L.fk_scar_raster(fake, fake, bad0, 1, 16, 16, fake, 16, fake, None) == 5
    short = (ctypes.c_int32 * 3)(0, 5, 7)  # a polygon of two vertices
    assert L.fk_scar_raster(fake, fake, short, 2, 16, 16, fake, 16, fake, None) == 5
    big = (ctypes.c_int32 * 2)(0, 5000)
    assert L.fk_scar_raster(fake, fake, big, 1, 16, 16, fake, 16, fake, None) == 5
    assert L.fk_conv2d_same(None, 8, 8, 8, fake, 3, fake + 64, 8, 0, None) == 1
    assert L.fk_conv2d_same(fake, 8, 8, 8, fake, 0, fake + 64, 8, 0, None) == 2
    assert L.fk_conv2d_same(fake, 8, 8, 4, fake, 3, fake + 64, 8, 0, None) == 2
    assert L.fk_conv2d_same(fake, 8, 8, 8, fake, 3, fake, 8, 0, None) == 5


def test_selftest_wait_timeout_checks_its_limit():
    from cardiax_gb300 import _native as N
    L = N.lib()
    assert L.fk_selftest_wait_timeout(10, None) == 5
    assert L.fk_selftest_wait_timeout(3_000_000_000, None) == 5

"""The C-ABI library loads on a machine without a GPU, exports every function that
include/c3d.h declares, and rejects bad arguments before touching a device."""
import ctypes
import os
import re

import pytest

from compact3d_gb300 import build, lib
from compact3d_gb300.grid import c3d_grid, make_grid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    build.build()
    return lib.load()


def declared():
    src = open(os.path.join(ROOT, "include", "c3d.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(c3d_[a-z_0-9]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(L):
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(lib.SIGNATURES), "Python signatures out of sync with c3d.h"


def test_schedule_length_agrees():
    """C3D_SCHEDULE_LEN in the header, the binding's constant and its knob names agree, so
    that a schedule dictionary maps onto the ints the library reads."""
    src = open(os.path.join(ROOT, "include", "c3d.h")).read()
    n = int(re.search(r"#define\s+C3D_SCHEDULE_LEN\s+(\d+)", src).group(1))
    assert n == lib.C3D_SCHEDULE_LEN == len(lib.Channel.SCHEDULE_KEYS)
    assert len(set(lib.Channel.SCHEDULE_KEYS)) == n


def test_error_strings(L):
    for code in (0, -1, -2, -3, -4, -5, -6, -7, -8, -99):
        assert L.c3d_error_string(code)


def test_version(L):
    assert L.c3d_version() >= 10000


@pytest.mark.parametrize("bad", [dict(n1m=50), dict(n3m=40), dict(n2m=2), dict(n1m=10)])
def test_create_rejects_bad_extents(L, bad):
    g, _ = make_grid("small32", **bad) if "n2m" not in bad or bad["n2m"] > 3 else (None, None)
    if g is None:
        g, _ = make_grid("small32")
        s = g.struct()
        s.n2 = 3
    else:
        s = g.struct()
    h = ctypes.c_void_p()
    assert L.c3d_create(ctypes.byref(s), ctypes.byref(h)) == -1
    assert L.c3d_last_error()


def test_create_rejects_null_metrics(L):
    g, _ = make_grid("small32")
    s = g.struct()
    s.hp = None
    h = ctypes.c_void_p()
    assert L.c3d_create(ctypes.byref(s), ctypes.byref(h)) == -1


def test_create_rejects_bad_precision_and_models(L):
    g, _ = make_grid("small32")
    for field, val in (("precision", 7), ("files", 4), ("re", -1.0), ("wmodel", 6), ("wmodel", -1)):
        s = g.struct()
        setattr(s, field, val)
        h = ctypes.c_void_p()
        assert L.c3d_create(ctypes.byref(s), ctypes.byref(h)) == -1


def test_null_handles(L):
    assert L.c3d_create(None, None) == -1
    assert L.c3d_step(None, 1, 0.001, None, None) == -1
    assert L.c3d_destroy(None) == -1
    assert L.c3d_upload(None, None, None, None, None) == -1
    assert L.c3d_diagnose(None, None) == -1
    assert L.c3d_batch_step(None, 1, None, None, None) == -1
    assert L.c3d_sync(None) == -1
    assert L.c3d_checkpoint_write(None, b"x", 1, 0.0, 0.0, 0.0) == -1
    assert L.c3d_checkpoint_read(None, b"x", None, None, None, None) == -1


def test_werner_needs_n3_not_above_n1(L):
    """WMODEL 4 (WALLMODEL_WERNER) indexes x with the z index, as the reference does;
    grids with N3M > N1M are refused before any device work."""
    g, _ = make_grid("les32cs", wmodel=4, n3m=64)
    s = g.struct()
    h = ctypes.c_void_p()
    assert L.c3d_create(ctypes.byref(s), ctypes.byref(h)) == -1


def test_shifted_wall_models_check_the_y_faces(L):
    """WMODEL 3 / 5 (MARUSIC1 / PIOMELLI) search the Y faces for the interpolation cell,
    so Y(1:N2) must increase; PIOMELLI's H(1) must lie within 2e-3 of YC(1) (its height
    climbs by 1e-6 per wall point below YC(1)).  Both are refused before any device work."""
    for wmodel in (3, 5):
        g, _ = make_grid("les32cs", wmodel=wmodel)
        g.arrays["y"][4] = g.arrays["y"][3]
        s = g.struct()
        h = ctypes.c_void_p()
        assert L.c3d_create(ctypes.byref(s), ctypes.byref(h)) == -1
        assert b"increase" in L.c3d_last_error()
    g, _ = make_grid("les32cs", wmodel=5, y0=0.01)
    s = g.struct()
    h = ctypes.c_void_p()
    assert L.c3d_create(ctypes.byref(s), ctypes.byref(h)) == -1
    assert b"H(1)" in L.c3d_last_error()


def test_rough_models_need_y0_below_the_sample_height(L):
    """Y(0) = Y0 != 0 selects the rough-wall models (WMODEL 1: WALLMODEL_ROUGH, 2:
    WALLMODEL_IWMLES_ROUGH), whose log(DELTAP / Y0) needs 0 < Y0 < DY(1)+DY(2)+DY(3)/2."""
    for wmodel, name in ((1, b"WALLMODEL_ROUGH"), (2, b"IWMLES_ROUGH")):
        g, _ = make_grid("les32cs", wmodel=wmodel, y0=-0.01)
        s = g.struct()
        h = ctypes.c_void_p()
        assert L.c3d_create(ctypes.byref(s), ctypes.byref(h)) == -1
        assert name in L.c3d_last_error()

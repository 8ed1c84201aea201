"""The allocation-free divergence check against the channel path.

c3d_divcheck_noalloc serves drivers that may not allocate device memory (their device
memory belongs to their own pool allocator, or their footprint must stay fixed after
start-up).  It works out of a static device array instead of cudaMalloc, so this test
checks that it gives DIVCHECK's max|div u| exactly as c3d_diagnose does on a channel, on
two calls in a row (a strongly divergent field first, then a projected one, so a running
maximum left over from the first call would show), and that a grid too large for the
static array is refused, and that repeated calls leave the device's free memory exactly
where it was (a cudaMalloc inside the call would lower it).  This file is collected last
on purpose.
"""
import ctypes

import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import C3D_FP64, make_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from compact3d_gb300 import build, lib
    build.build()
    return lib


def noalloc_divmax(L, g, U):
    s = g.struct()
    out = (ctypes.c_double * 1)()
    rc = L.load().c3d_divcheck_noalloc(ctypes.byref(s), U.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out)
    L.check(rc, "c3d_divcheck_noalloc")
    return out[0]


def channel_divmax(L, g, U):
    ch = L.Channel(g, C3D_FP64)
    ch.upload(U, g.zeros_p(), g.zeros_u())
    d = ch.diagnose()["divmax"]
    ch.close()
    return d


@pytest.mark.parametrize("name", ["small32", "channel64"])
def test_noalloc_matches_channel_two_calls(L, name):
    g, _ = make_grid(name)
    Ua, _, _ = ic.perturbed_laminar(g, seed=5)          # not projected: |div| ~ 1e-3
    Ub = Ua.copy(order="F")
    ch = L.Channel(g, C3D_FP64)
    ch.upload(Ub, g.zeros_p(), g.zeros_u())
    ch.project()
    Ub, _, _ = ch.download(Ub)                           # projected: |div| ~ 1e-14
    ch.close()
    ref_a = channel_divmax(L, g, Ua)
    ref_b = channel_divmax(L, g, Ub)
    assert ref_a > 1e-6 and ref_b < 1e-11
    got_a = noalloc_divmax(L, g, Ua)
    got_b = noalloc_divmax(L, g, Ub)
    assert got_a == pytest.approx(ref_a, rel=1e-12)
    assert got_b == pytest.approx(ref_b, rel=1e-9, abs=1e-15)


def test_noalloc_rejects_oversize_grid(L):
    g, _ = make_grid("channel384")
    U = np.zeros(g.shape_u(), order="F")
    s = g.struct()
    out = (ctypes.c_double * 1)()
    rc = L.load().c3d_divcheck_noalloc(ctypes.byref(s), U.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out)
    assert rc == -1
    assert b"too large" in L.load().c3d_last_error()


def test_noalloc_allocates_nothing(L):
    """After a first call (which looks up the scratch address and loads the kernels),
    five more calls leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    g, _ = make_grid("channel64")
    U, _, _ = ic.perturbed_laminar(g, seed=7)
    L.check(L.load().c3d_set_device(0), "c3d_set_device")
    torch.cuda.mem_get_info(0)
    first = noalloc_divmax(L, g, U)
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(5):
        assert noalloc_divmax(L, g, U) == first
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)

"""c3d_getup with host arrays registered (mapped, transfers of HH overlapping the step) and
unregistered (staged copies around the step): the same kernels in the same order on the
device, so the host arrays after each call are bitwise equal, and equal to c3d_upload +
c3d_step + c3d_download; the LES form returns SGSVIS the same way."""
import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, make_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libc3d():
    from compact3d_gb300 import build, lib
    build.build()
    lib.load()
    return lib


def _run(lib, g, dt, U0, P0, HH0, register, steps=3, sgs=False):
    U, P, HH = U0.copy(order="F"), P0.copy(order="F"), HH0.copy(order="F")
    S = np.zeros(U.shape[:3], order="F") if sgs else None
    arrs = [U, P, HH] + ([S] if sgs else [])
    if register:
        for a in arrs:
            lib.host_register(a)
    ch = lib.Channel(g, g.precision)
    pg = pg3 = 0.0
    try:
        for m in range(1, steps + 1):
            pg, pg3 = ch.getup(U, P, HH, m, dt, pg, pg3, sgsvis=S)
    finally:
        ch.close()
        if register:
            for a in arrs:
                lib.host_unregister(a)
    return U, P, HH, S, pg, pg3


@pytest.mark.parametrize("prec", [C3D_FP64, C3D_MIXED])
def test_getup_mapped_equals_staged(libc3d, prec):
    g, dt = make_grid("small32", prec, n1m=64, n2m=32, n3m=64)
    U0, P0, HH0 = ic.perturbed_laminar(g)
    a = _run(libc3d, g, dt, U0, P0, HH0, True)
    b = _run(libc3d, g, dt, U0, P0, HH0, False)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert a[4] == b[4] and a[5] == b[5]


def test_getup_mapped_equals_step_path(libc3d):
    # FP64: the host arrays carry the state exactly, so re-uploading it every step changes
    # nothing (a double-float state may come back as another pair for the same value)
    g, dt = make_grid("small32", C3D_FP64, n1m=64, n2m=32, n3m=64)
    U0, P0, HH0 = ic.perturbed_laminar(g)
    a = _run(libc3d, g, dt, U0, P0, HH0, True, steps=2)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U0, P0, HH0)
    pg = pg3 = 0.0
    for m in (1, 2):
        pg, pg3 = ch.step(m, dt, pg, pg3)
    U, P, HH = ch.download()
    ch.close()
    for x, y in zip(a[:3], (U, P, HH)):
        assert np.array_equal(x, y)


def test_getup_mapped_les_sgsvis(libc3d):
    g, dt = make_grid("les32cs")
    U0, P0, HH0 = ic.loglaw(g, 395.0, 0.05, 7)
    a = _run(libc3d, g, dt, U0, P0, HH0, True, steps=2, sgs=True)
    b = _run(libc3d, g, dt, U0, P0, HH0, False, steps=2, sgs=True)
    for x, y in zip(a[:4], b[:4]):
        assert np.array_equal(x, y)
    assert np.abs(a[3]).max() > 0.0


def test_getup_host_alloc_arrays(libc3d):
    """Arrays in page-locked memory from c3d_host_alloc take the DMA path of registered
    arrays: c3d_getup on them gives the device-resident step bit for bit (FP64)."""
    g, dt = make_grid("small32", C3D_FP64, n1m=64, n2m=32, n3m=64)
    U0, P0, HH0 = ic.perturbed_laminar(g)
    U, P, HH = (libc3d.host_array(a.shape) for a in (U0, P0, HH0))
    U[...], P[...], HH[...] = U0, P0, HH0
    ch = libc3d.Channel(g, C3D_FP64)
    pg = pg3 = 0.0
    for m in (1, 2):
        pg, pg3 = ch.getup(U, P, HH, m, dt, pg, pg3)
    ch.close()
    ref = libc3d.Channel(g, C3D_FP64)
    ref.upload(U0, P0, HH0)
    qg = qg3 = 0.0
    for m in (1, 2):
        qg, qg3 = ref.step(m, dt, qg, qg3)
    for x, y in zip((U, P, HH), ref.download()):
        assert np.array_equal(x, y)
    ref.close()
    for a in (U, P, HH):
        libc3d.host_free(a)


def test_getup_concurrent_pieces(libc3d):
    """c3d_getup on page-locked arrays with the explicit pieces as concurrent branches
    (knob 15): the upload of HH_old on the side stream, the pieces on the two extra
    streams and the download of the new HH after xB keep their order, so the host arrays
    equal the device-resident step with the pieces one after another, bit for bit (FP64)."""
    g, dt = make_grid("small32", C3D_FP64, n1m=64, n2m=32, n3m=64)
    U0, P0, HH0 = ic.perturbed_laminar(g)
    U, P, HH = (libc3d.host_array(a.shape) for a in (U0, P0, HH0))
    U[...], P[...], HH[...] = U0, P0, HH0
    ch = libc3d.Channel(g, C3D_FP64)
    ch.set_schedule(dict(ch.get_schedule(), x_split_xA=1, z_split_zA=1, concurrent_pieces=1))
    pg = pg3 = 0.0
    for m in (1, 2, 3):
        pg, pg3 = ch.getup(U, P, HH, m, dt, pg, pg3)
    ch.close()
    ref = libc3d.Channel(g, C3D_FP64)
    ref.set_schedule(dict(ref.get_schedule(), x_split_xA=1, z_split_zA=1, concurrent_pieces=0))
    ref.upload(U0, P0, HH0)
    qg = qg3 = 0.0
    for m in (1, 2, 3):
        qg, qg3 = ref.step(m, dt, qg, qg3)
    for x, y in zip((U, P, HH), ref.download()):
        assert np.array_equal(x, y)
    assert pg == qg and pg3 == qg3
    ref.close()
    for a in (U, P, HH):
        libc3d.host_free(a)


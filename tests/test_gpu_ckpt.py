"""Checkpoints written from and read into the device state (c3d_checkpoint_write/read):
the bytes equal the format restated in numpy (tests/ckpt_format.py) for the downloaded
fields, and a channel restarted from a checkpoint continues bit for bit (FP64; the mixed
form's double-float state comes back as the same values)."""
import os

import numpy as np
import pytest

import ckpt_format as F
from compact3d_gb300 import ic
from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, make_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libc3d():
    from compact3d_gb300 import build, lib
    build.build()
    lib.load()
    return lib


def _run(lib, g, dt, prec, steps=2, sgs=False):
    U, P, HH = (ic.loglaw(g, 2000.0) if sgs else ic.perturbed_laminar(g))
    ch = lib.Channel(g, prec)
    ch.upload(U, P, HH)
    ch.project()
    pg = pg3 = 0.0
    for m in range(1, steps + 1):
        pg, pg3 = ch.step(m, dt, pg, pg3)
    return ch, pg, pg3


@pytest.mark.parametrize("prec", [C3D_FP64, C3D_MIXED])
def test_checkpoint_bytes_and_exact_restart(libc3d, tmp_path, prec):
    g, dt = make_grid("small32", n1m=64, n2m=32, n3m=64)
    ch, pg, pg3 = _run(libc3d, g, dt, prec)
    path = tmp_path / "ckpt.bin"
    ch.checkpoint_write(path, 2, 2 * dt, pg, pg3)
    U, P, HH = ch.download()
    ref = F.records(g.n1m, g.n2m, g.n3m, pg, pg3, 2, 2 * dt, U, P, HH)
    data = path.read_bytes()
    assert data == ref
    # restart into a fresh channel and continue both
    r = libc3d.Channel(g, prec)
    nt, tm, pga, pg3a = r.checkpoint_read(path)
    assert (nt, tm, pga, pg3a) == (2, 2 * dt, pg, pg3)
    a = (pg, pg3)
    b = (pga, pg3a)
    for m in (3, 4):
        a = ch.step(m, dt, *a)
        b = r.step(m, dt, *b)
    for x, y in zip(ch.download(), r.download()):
        if prec == C3D_FP64:
            assert np.array_equal(x, y)
        else:
            assert np.linalg.norm(x - y) <= 1e-13 * np.linalg.norm(y)
    assert a == b if prec == C3D_FP64 else np.allclose(a, b, rtol=1e-12, atol=1e-18)


def test_checkpoint_les_wall_state(libc3d, tmp_path):
    g, dt = make_grid("les32cs")
    ch, pg, pg3 = _run(libc3d, g, dt, C3D_FP64, sgs=True)
    path = tmp_path / "les.bin"
    ch.checkpoint_write(path, 2, 0.0, pg, pg3)
    recs = F.split(path.read_bytes())
    assert len(recs) == 8
    tw, tb = ch.download_wall()
    w = np.frombuffer(recs[7], "<f8")
    assert np.array_equal(w[:tw.size], tw.ravel(order="F")) and np.array_equal(w[-3:], ch.get_wsm())
    r = libc3d.Channel(g, C3D_FP64)
    _, _, pga, pg3a = r.checkpoint_read(path)
    a, b = (pg, pg3), (pga, pg3a)
    for m in (3, 4):
        a = ch.step(m, dt, *a)
        b = r.step(m, dt, *b)
    for x, y in zip(ch.download(), r.download()):
        assert np.array_equal(x, y)


def test_checkpoint_errors(libc3d, tmp_path):
    g, dt = make_grid("small32")
    ch, pg, pg3 = _run(libc3d, g, dt, C3D_FP64, steps=1)
    path = tmp_path / "c.bin"
    ch.checkpoint_write(path, 1, 0.0, pg, pg3)
    other, _ = make_grid("small32", n3m=64)
    with pytest.raises(libc3d.C3DError) as e:
        libc3d.Channel(other, C3D_FP64).checkpoint_read(path)
    assert e.value.code == -1
    cut = tmp_path / "cut.bin"
    cut.write_bytes(path.read_bytes()[:-100])
    with pytest.raises(libc3d.C3DError) as e:
        libc3d.Channel(g, C3D_FP64).checkpoint_read(cut)
    assert e.value.code == -8
    with pytest.raises(libc3d.C3DError) as e:
        ch.checkpoint_read(os.path.join(str(tmp_path), "missing.bin"))
    assert e.value.code == -8
    # a file cut inside the P record and one with a bad HH record marker: refused before
    # any of the channel's state is replaced (the state downloads unchanged and steps on)
    before = ch.download()
    nu = 3 * g.n1m * (g.n2m + 2) * g.n3m
    np_ = g.n1m * g.n2m * g.n3m
    p_start = (12 + 8) + (16 + 8) + (4 + 8) + (8 + 8) + (nu * 8 + 8)
    raw = path.read_bytes()
    cut_p = tmp_path / "cut_p.bin"
    cut_p.write_bytes(raw[:p_start + 4 + np_ * 4])
    bad_hh = bytearray(raw)
    hh_start = p_start + np_ * 8 + 8
    bad_hh[hh_start:hh_start + 4] = (12345).to_bytes(4, "little")
    bad = tmp_path / "bad_hh.bin"
    bad.write_bytes(bytes(bad_hh))
    for f in (cut_p, bad):
        with pytest.raises(libc3d.C3DError) as e:
            ch.checkpoint_read(f)
        assert e.value.code == -8
        after = ch.download()
        for x, y in zip(before, after):
            assert np.array_equal(x, y)
    ch.step(2, dt, pg, pg3)

"""Batched ensemble: channels of different sizes, Reynolds numbers and precisions stepped
together as one CUDA graph give exactly the results of stepping each channel alone."""
import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, Grid, make_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from compact3d_gb300 import build, lib
    build.build()
    return lib


def ensemble():
    specs = [("tiny16", C3D_FP64, {}), ("small32", C3D_MIXED, dict(re=3000.0)),
             ("channel64", C3D_MIXED, dict(n1m=48, n3m=96, n2m=48, re=6000.0)),
             ("small32", C3D_FP64, dict(n1m=64, n2m=32, n3m=64))]
    out = []
    for i, (name, prec, over) in enumerate(specs):
        g, dt = make_grid(name, precision=prec, **over)
        out.append((g, dt, ic.perturbed_laminar(g, seed=ic.SEED0 + i)))
    return out


def test_batch_matches_single_channels(L):
    ens = ensemble()
    b = L.Batch([g for g, _, _ in ens])
    singles = []
    for (g, dt, (U, P, HH)), ch in zip(ens, b.channels):
        ch.upload(U, P, HH)
        ch.project()
        s = L.Channel(g)
        s.upload(U, P, HH)
        s.project()
        singles.append(s)
    dts = [dt for _, dt, _ in ens]
    pb, pb3 = [0.0] * len(ens), [0.0] * len(ens)
    ps = [(0.0, 0.0) for _ in ens]
    for n in range(1, 6):
        pb, pb3 = b.step(n, dts, pb, pb3)
        ps = [s.step(n, dt, *p) for s, dt, p in zip(singles, dts, ps)]
    for i, ((g, _, _), ch, s) in enumerate(zip(ens, b.channels, singles)):
        Ub, Pb, Hb = ch.download()
        Us, Ps, Hs = s.download()
        assert np.array_equal(Ub, Us), i
        assert np.array_equal(Pb, Ps), i
        assert np.array_equal(Hb, Hs), i
        assert pb[i] == ps[i][0] and pb3[i] == ps[i][1]
    ms, nl = b.last_step_stats()
    assert ms > 0 and nl >= 15 * len(ens)
    for s in singles:
        s.close()
    b.close()


def test_batch_dt_change_recaptures(L):
    ens = ensemble()[:2]
    b = L.Batch([g for g, _, _ in ens])
    ref = []
    for (g, dt, (U, P, HH)), ch in zip(ens, b.channels):
        ch.upload(U, P, HH)
        s = L.Channel(g)
        s.upload(U, P, HH)
        ref.append(s)
    p, p3 = [0.0, 0.0], [0.0, 0.0]
    r = [(0.0, 0.0), (0.0, 0.0)]
    for n, scale in enumerate([1.0, 1.0, 0.5, 0.5, 1.0], start=1):
        dts = [dt * scale for _, dt, _ in ens]
        p, p3 = b.step(n, dts, p, p3)
        r = [s.step(n, d, *q) for s, d, q in zip(ref, dts, r)]
    for ch, s in zip(b.channels, ref):
        assert np.array_equal(ch.download()[0], s.download()[0])
        s.close()
    b.close()


def test_batch_of_les_channels_matches_single_channels(L):
    """LES channels in a batch graph, whose wall models and SGSSD root solve run on side
    streams forked and joined inside each channel's step: bitwise the single steps."""
    specs = [("les32cs", C3D_FP64, dict(wmodel=3)), ("les32dy", C3D_FP64, dict(files=3)),
             ("les32cs", C3D_MIXED, dict(wmodel=1)), ("les32dy", C3D_MIXED, dict(wmodel=5))]
    ens = []
    for i, (name, prec, over) in enumerate(specs):
        g, dt = make_grid(name, precision=prec, **over)
        ens.append((g, dt, ic.loglaw(g, 2000.0, seed=ic.SEED0 + i)))
    b = L.Batch([g for g, _, _ in ens])
    singles = []
    for (g, dt, (U, P, HH)), ch in zip(ens, b.channels):
        for c in (ch, None):
            s = c or L.Channel(g)
            s.upload(U, P, HH)
            s.project()
            if c is None:
                singles.append(s)
    dts = [dt for _, dt, _ in ens]
    pb, pb3 = [0.0] * len(ens), [0.0] * len(ens)
    ps = [(0.0, 0.0) for _ in ens]
    for n in range(1, 5):
        pb, pb3 = b.step(n, dts, pb, pb3)
        ps = [s.step(n, dt, *p) for s, dt, p in zip(singles, dts, ps)]
    for i, (ch, s) in enumerate(zip(b.channels, singles)):
        for x, y in zip(ch.download(), s.download()):
            assert np.array_equal(x, y), i
        for x, y in zip(ch.download_wall(), s.download_wall()):
            assert np.array_equal(x, y), i
    for s in singles:
        s.close()
    b.close()


def test_batch_refuses_iwmles(L):
    g, _ = make_grid("les32cs", wmodel=2)
    with pytest.raises(L.C3DError):
        L.Batch([g])

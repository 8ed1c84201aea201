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


@pytest.mark.parametrize("groups", [1, 2])
def test_worklist_concurrent_pieces_bit_identical(L, groups):
    """The work-list form with the pieces of xA and zA as concurrent branches of each group
    against the same form with the pieces one after another (the default): the same
    kernels on the same data, disjoint outputs, so every channel's state is bitwise equal."""
    ens = dns_ensemble(C3D_MIXED)
    res = []
    for conc in (0, 1):
        b = L.Batch([g for g, _, _ in ens])
        for (g, dt, (U, P, HH)), ch in zip(ens, b.channels):
            ch.upload(U, P, HH)
        b.set_groups(groups)
        b.set_concurrent(conc)
        dts = [dt for _, dt, _ in ens]
        p, p3 = [0.0] * len(ens), [0.0] * len(ens)
        for n in range(1, 4):
            p, p3 = b.step(n, dts, p, p3)
        res.append([ch.download() for ch in b.channels] + [p])
        b.close()
    for x, y in zip(res[0][:-1], res[1][:-1]):
        for a, c in zip(x, y):
            assert np.array_equal(a, c)
    assert res[0][-1] == res[1][-1]


def test_streams_form_with_concurrent_pieces(L):
    """Channels whose explicit pieces run as concurrent branches (schedule knob 15) inside
    the streams form's graph: the forks onto each channel's extra streams are captured with
    its step, and the results are bitwise those of single channels that run the pieces one
    after another."""
    ens = dns_ensemble(C3D_MIXED)[:3]
    b = L.Batch([g for g, _, _ in ens])
    b.set_form("streams")
    singles = []
    for (g, dt, (U, P, HH)), ch in zip(ens, b.channels):
        ch.upload(U, P, HH)
        ch.set_schedule(dict(ch.get_schedule(), x_split_xA=1, z_split_zA=1, concurrent_pieces=1))
        s = L.Channel(g)
        s.upload(U, P, HH)
        s.set_schedule(dict(s.get_schedule(), x_split_xA=1, z_split_zA=1, concurrent_pieces=0))
        singles.append(s)
    dts = [dt for _, dt, _ in ens]
    pb, pb3 = [0.0] * len(ens), [0.0] * len(ens)
    ps = [(0.0, 0.0) for _ in ens]
    for n in range(1, 4):
        pb, pb3 = b.step(n, dts, pb, pb3)
        ps = [s.step(n, dt, *p) for s, dt, p in zip(singles, dts, ps)]
    for i, (ch, s) in enumerate(zip(b.channels, singles)):
        for x, y in zip(ch.download(), s.download()):
            assert np.array_equal(x, y), i
    for s in singles:
        s.close()
    b.close()


def test_batch_refuses_iwmles(L):
    g, _ = make_grid("les32cs", wmodel=2)
    with pytest.raises(L.C3DError):
        L.Batch([g])


def row_lanes(g):
    """Lanes per row of the work-list form's xA pieces and xB: 8 for rows of 48, 64 or
    96 points, 16 for 128 (when N3M is a multiple of 32 / lanes), else a warp (0)."""
    w = {48: 8, 64: 8, 96: 8, 128: 16}.get(g.n1m, 0)
    return w if w and g.n3m % (32 // w) == 0 else 0


WORKLIST_Z = (8, 8, 16, 16, 8)   # default z segment lengths of zA..zE in the work-list form


def worklist_schedule(ch, g, zseg=WORKLIST_Z, xw=2):
    """The fixed schedule of the work-list form (include/c3d.h) on a single channel."""
    s = ch.get_schedule()
    s.update({f"z_segment_z{c}": (L if g.n3m % L == 0 else 16) for c, L in zip("ABCDE", zseg)})
    s.update(x_rows_per_block=xw, fft_z_tile=0, fft_x_plan=3 if g.n1m % 64 == 0 else 0, fft_z_plan=0,
             z_split_zA=1, x_split_xA=1, x_bulk_stages=0, x_stage_xA=0, x_row_lanes=row_lanes(g))
    ch.set_schedule(s)


def dns_ensemble(prec, seed0=0):
    """DNS channels of one precision covering the lane chunks and z-FFT forms the
    work-list form groups by: N1M in {48, 64, 96, 128}, N3M in {48, 64, 96, 128}."""
    shapes = [(48, 32, 64), (64, 48, 48), (96, 40, 96), (128, 24, 128), (48, 64, 96), (64, 32, 64)]
    out = []
    for i, (n1, n2, n3) in enumerate(shapes):
        g, dt = make_grid("channel64", precision=prec, n1m=n1, n2m=n2, n3m=n3, re=3000.0 + 700.0 * i)
        out.append((g, dt, ic.perturbed_laminar(g, seed=ic.SEED0 + seed0 + i)))
    return out


@pytest.mark.parametrize("prec,zseg,xw", [(C3D_MIXED, WORKLIST_Z, 2), (C3D_FP64, WORKLIST_Z, 2),
                                          (C3D_FP64, (32, 16, 8, 32, 16), 8)])
def test_worklist_batch_matches_single_channels(L, prec, zseg, xw):
    """One launch per pass over all channels (the work-list form) computes, for every
    channel, the step of that channel alone under the same schedule.  The batch kernels
    are other compiled instances of the same kernel bodies, whose multiply-add
    contractions can differ in the last bit, so after five steps they agree to rounding:
    FP64 1e-12 relative (P 1e-11), mixed 1e-8 for U, 1e-4 for HH and 1e-3 for P (the
    mixed pressure amplifies FP32 rounding, as its error against FP64 shows)."""
    ens = dns_ensemble(prec)
    b = L.Batch([g for g, _, _ in ens])
    assert b.get_form() == "worklist"
    if zseg != WORKLIST_Z:   # segment lengths a channel cannot take (32 on N3M = 48) run 16
        b.set_z_segments(zseg)
    if xw != 2:
        b.set_x_warps(xw)
    singles = []
    for (g, dt, (U, P, HH)), ch in zip(ens, b.channels):
        ch.upload(U, P, HH)
        ch.project()
        s = L.Channel(g)
        s.upload(U, P, HH)
        s.project()
        worklist_schedule(s, g, zseg, xw)
        singles.append(s)
    dts = [dt for _, dt, _ in ens]
    pb, pb3 = [0.0] * len(ens), [0.0] * len(ens)
    ps = [(0.0, 0.0) for _ in ens]
    for n in range(1, 6):
        pb, pb3 = b.step(n, dts, pb, pb3)
        ps = [s.step(n, dt, *p) for s, dt, p in zip(singles, dts, ps)]
    tol = (1e-12, 1e-11, 1e-12) if prec == C3D_FP64 else (1e-8, 1e-3, 1e-4)
    for i, (ch, s) in enumerate(zip(b.channels, singles)):
        for f, x, y, t_ in zip("UPH", ch.download(), s.download(), tol):
            e = float(np.linalg.norm(x - y) / np.linalg.norm(y))
            assert e < t_, (i, f, e)
        assert pb[i] == pytest.approx(ps[i][0], rel=1e-9 if prec == C3D_FP64 else 1e-6)
    ms, nl = b.last_step_stats()
    # 20 passes per channel group (two by default), a few kernel groups for the x and FFT
    # passes: tens of launches against one step's 15-20 per channel in the streams form
    assert ms > 0 and nl <= 100
    for s in singles:
        s.close()
    b.close()


def test_worklist_batch_fp64_matches_oracle(L, oracle_mod):
    """The work-list form in FP64 against the oracle, two steps per channel, 1e-10."""
    ens = dns_ensemble(C3D_FP64, seed0=10)[:4]
    b = L.Batch([g for g, _, _ in ens])
    orcs = []
    for (g, dt, (U, P, HH)), ch in zip(ens, b.channels):
        o = oracle_mod.Oracle(g)
        o.project(U)
        ch.upload(U, P, HH)
        orcs.append((o, U, P, HH))
    dts = [dt for _, dt, _ in ens]
    pb, pb3 = [0.0] * len(ens), [0.0] * len(ens)
    po = [(0.0, 0.0) for _ in ens]
    for n in (1, 2):
        pb, pb3 = b.step(n, dts, pb, pb3)
        po = [o.getup(U, P, HH, n, dt, *p) for (o, U, P, HH), dt, p in zip(orcs, dts, po)]
    for i, ((g, _, _), ch, (o, U, P, HH)) in enumerate(zip(ens, b.channels, orcs)):
        Ug, Pg, Hg = ch.download()
        n1, n2, n3 = g.n1m, g.n2m, g.n3m
        for c, j0 in ((0, 1), (1, 2), (2, 1)):
            a = Ug[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c]
            r = U[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c]
            assert np.linalg.norm(a - r) / np.linalg.norm(r) < 1e-10, (i, c)
        assert pb[i] == pytest.approx(po[i][0], rel=1e-9)
    b.close()


def test_mixed_precision_batch_runs_streams_form(L):
    ens = ensemble()
    b = L.Batch([g for g, _, _ in ens])
    assert b.get_form() == "streams"            # FP64 and mixed channels together
    b.close()
    ens = dns_ensemble(C3D_MIXED)[:2]
    b = L.Batch([g for g, _, _ in ens])
    b.set_form("streams")
    assert b.get_form() == "streams"
    b.set_form("worklist")
    assert b.get_form() == "worklist"
    with pytest.raises(L.C3DError):
        b.set_z_segments([12, 16, 16, 16, 16])
    with pytest.raises(L.C3DError):
        b.set_x_warps(3)
    with pytest.raises(L.C3DError):
        b.set_concurrent(2)
    b.close()

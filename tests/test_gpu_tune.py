"""Launch schedules: every schedule the autotuner can choose computes the same step.

Each schedule knob (z segment length, x rows per block, z-FFT tile width, x/z FFT radix
order) changes only the order of floating-point operations, so one FP64 step under any
schedule stays within the parity tolerance of the FP64 oracle (1e-10 relative L2 for
U, V, W).  The autotuner returns a valid schedule and caches it per grid shape.
"""
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


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _sched(zl, xw, tw, fx, fz, split, xsplit, xbulk=0, xstage=0, ycn=0, xlanes=0, conc=0):
    d = {f"z_segment_z{c}": z for c, z in zip("ABCDE", zl)}
    d.update(x_rows_per_block=xw, fft_z_tile=tw, fft_x_plan=fx, fft_z_plan=fz, z_split_zA=split,
             x_split_xA=xsplit, x_bulk_stages=xbulk, x_stage_xA=xstage, ycn_tile=ycn, x_row_lanes=xlanes,
             concurrent_pieces=conc)
    return d


# (schedule, N3M); z segment length 0 is the block form (segments of 8 points for N3M = 64,
# 12 points in 32 segments for N3M = 384); z-FFT tile 0 is the four-step warp FFT
# (N1 = N3M / 32 = 2 and 12 points per lane)
SCHEDULES = [
    (_sched((8, 8, 8, 8, 8), 2, 4, 1, 2, 1, 1), 64),
    (_sched((32, 32, 32, 32, 32), 8, 16, 2, 1, 0, 0), 64),
    (_sched((16, 8, 32, 16, 8), 4, 8, 0, 0, 1, 0, 2), 64),
    (_sched((0, 0, 0, 0, 0), 2, 0, 0, 1, 1, 1), 64),
    (_sched((0, 0, 0, 0, 0), 2, 0, 0, 1, 0, 0), 384),
    (_sched((16, 16, 16, 16, 16), 2, 0, 0, 1, 1, 1), 96),
    (_sched((8, 8, 32, 16, 8), 2, 0, 2, 1, 1, 1), 64),
    (_sched((16, 8, 32, 16, 8), 4, 0, 2, 1, 1, 1, 0, 1), 64),
    (_sched((16, 16, 16, 16, 16), 2, 0, 0, 1, 1, 1, 0, 0, 32), 64),
    (_sched((16, 16, 16, 16, 16), 2, 0, 0, 1, 1, 1, 0, 0, 64), 96),
]


@pytest.mark.parametrize("n1m", [64, 128, 192, 256, 384])
def test_register_row_fft_matches_oracle(libc3d, oracle_mod, n1m):
    """The four-step register row FFT (x plan 3) for every even N1M / 32: one FP64 step
    within 1e-10 of the oracle."""
    g, dt = make_grid("small32", n1m=n1m, n2m=16, n3m=32)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    s = ch.get_schedule()
    s.update(fft_x_plan=3)
    ch.set_schedule(s)
    orc.getup(U, P, HH, 1, dt, 0.0, 0.0)
    ch.step(1, dt, 0.0, 0.0)
    Ug, Pg, _ = ch.download()
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    for c, j0 in ((0, 1), (1, 2), (2, 1)):
        e = rel(Ug[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c], U[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c])
        assert e < 1e-10, (n1m, c, e)


@pytest.mark.parametrize("n1m", [48, 96])
def test_x_plan3_refused_unless_n1m_multiple_of_64(libc3d, oracle_mod, n1m):
    """The register row FFT needs all 32 lanes to hold an even chunk: for N1M = 48 or 96
    the schedule is refused, and the tuned step of such a grid matches the oracle."""
    g, dt = make_grid("small32", n1m=n1m, n2m=16, n3m=32)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    s = ch.get_schedule()
    with pytest.raises(libc3d.C3DError):
        ch.set_schedule(dict(s, fft_x_plan=3))
    assert ch.autotune()["fft_x_plan"] != 3
    orc.getup(U, P, HH, 1, dt, 0.0, 0.0)
    ch.step(1, dt, 0.0, 0.0)
    Ug, _, _ = ch.download()
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    for c, j0 in ((0, 1), (1, 2), (2, 1)):
        e = rel(Ug[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c], U[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c])
        assert e < 1e-10, (n1m, c, e)


@pytest.mark.parametrize("n1m,lanes", [(48, 8), (64, 8), (96, 8), (128, 16)])
def test_row_segments_match_oracle(libc3d, oracle_mod, n1m, lanes):
    """xA's pieces and xB with a row per segment of 8 or 16 lanes (4 or 2 rows per warp,
    6 to 12 points per lane): one FP64 step within 1e-10 of the oracle; the mixed form
    within FP32 rounding of its whole-warp step; other lane counts are refused."""
    g, dt = make_grid("small32", n1m=n1m, n2m=16, n3m=32)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    s = ch.get_schedule()
    s.update(x_split_xA=1, x_stage_xA=0, x_row_lanes=lanes)
    ch.set_schedule(s)
    assert ch.get_schedule()["x_row_lanes"] == lanes
    with pytest.raises(libc3d.C3DError):
        ch.set_schedule(dict(s, x_row_lanes=24 - lanes))
    U0, P0, H0 = U.copy(order="F"), P.copy(order="F"), HH.copy(order="F")
    orc.getup(U, P, HH, 1, dt, 0.0, 0.0)
    ch.step(1, dt, 0.0, 0.0)
    Ug, _, Hg = ch.download()
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    for c, j0 in ((0, 1), (1, 2), (2, 1)):
        e = rel(Ug[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c], U[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c])
        assert e < 1e-10, (n1m, c, e)
    assert rel(Hg[1:n1 + 1, 1:n2 + 1, 1:n3 + 1], HH[1:n1 + 1, 1:n2 + 1, 1:n3 + 1]) < 1e-10
    ch.close()
    out = []
    for w in (0, lanes):
        m = libc3d.Channel(g, C3D_MIXED)
        m.upload(U0, P0, H0)
        m.set_schedule(dict(m.get_schedule(), x_split_xA=1, x_stage_xA=0, x_row_lanes=w))
        pg = pg3 = 0.0
        for n in (1, 2, 3):
            pg, pg3 = m.step(n, dt, pg, pg3)
        out.append(m.download())
        m.close()
    assert rel(out[1][0], out[0][0]) < 1e-8
    assert rel(out[1][2], out[0][2]) < 1e-4


@pytest.mark.parametrize("prec,xstage", [(C3D_MIXED, 0), (C3D_MIXED, 1), (C3D_FP64, 0)])
def test_concurrent_pieces_bit_identical(libc3d, prec, xstage):
    """The explicit pieces as concurrent branches (knob 15) run the same kernels on the same
    data in another order of launch; they write disjoint fields, so the step is
    bit-identical to the pieces one after another."""
    g, dt = make_grid("small32", n1m=64, n2m=24, n3m=64)
    U, P, HH = ic.perturbed_laminar(g)
    out = []
    for conc in (0, 1):
        ch = libc3d.Channel(g, prec)
        ch.upload(U, P, HH)
        ch.set_schedule(dict(ch.get_schedule(), x_split_xA=1, z_split_zA=1, x_stage_xA=xstage,
                             concurrent_pieces=conc))
        pg = pg3 = 0.0
        for m in (1, 2, 3):
            pg, pg3 = ch.step(m, dt, pg, pg3)
        out.append(ch.download() + (pg,))
        ch.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("sched,n3m", SCHEDULES)
def test_every_schedule_matches_oracle(libc3d, oracle_mod, sched, n3m):
    g, dt = make_grid("small32", n3m=n3m)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    pg = pg3 = 0.0
    pg, pg3 = orc.getup(U, P, HH, 1, dt, pg, pg3)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    ch.set_schedule(sched)
    assert ch.get_schedule() == sched
    orc.getup(U, P, HH, 2, dt, pg, pg3)
    ch.step(2, dt, pg, pg3)
    Ug, _, _ = ch.download()
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    for c, j0 in ((0, 1), (1, 2), (2, 1)):
        e = rel(Ug[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c], U[1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c])
        assert e < 1e-10, (sched, c, e)


def test_autotune_valid_and_cached(libc3d):
    g, dt = make_grid("channel64")
    U, P, HH = ic.perturbed_laminar(g)
    a = libc3d.Channel(g, C3D_MIXED)
    a.upload(U, P, HH)
    a.project()
    s1 = a.autotune()
    assert all(s1[f"z_segment_z{c}"] in (0, 8, 16, 32) for c in "ABCDE") and s1["x_rows_per_block"] in (2, 4, 8)
    assert s1["fft_z_tile"] in (0, 4, 8, 16) and s1["fft_x_plan"] in (0, 1, 2, 3) and s1["fft_z_plan"] in (0, 1, 2)
    b = libc3d.Channel(g, C3D_MIXED)
    b.upload(U, P, HH)
    assert b.autotune() == s1          # cached for the same grid shape and form
    a.step_async(1, dt)
    a.sync()
    d = a.diagnose()
    assert np.isfinite(d["divmax"]) and d["divmax"] < 1e-4
    with pytest.raises(libc3d.C3DError):
        a.set_schedule(dict(s1, z_segment_zA=12))


@pytest.mark.parametrize("shape,fxp", [((32, 128, 256), 0), ((96, 64, 64), 0), ((64, 128, 128), 3)])
def test_bulk_rows_bit_identical(libc3d, shape, fxp):
    """The bulk-copy ring only changes where a row is read from: the mixed step is
    bit-identical with 0, 2 or 3 stages.  (32, 128, 256) gives every persistent warp
    several rows, so each stage's barrier runs through several phases."""
    n1m, n2m, n3m = shape
    g, dt = make_grid("small32", n1m=n1m, n2m=n2m, n3m=n3m)
    U, P, HH = ic.perturbed_laminar(g)
    out = []
    for xb in (0, 2, 3):
        ch = libc3d.Channel(g, C3D_MIXED)
        ch.upload(U, P, HH)
        s = ch.get_schedule()
        s.update(x_bulk_stages=xb, fft_x_plan=fxp)
        ch.set_schedule(s)
        for m in (1, 2, 3):
            ch.step(m, dt, 0.0, 0.0)
        out.append(ch.download())
        ch.close()
    for r in out[1:]:
        for a, b in zip(r, out[0]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("n1m,prec", [(32, C3D_MIXED), (96, C3D_MIXED), (384, C3D_MIXED), (64, C3D_FP64),
                                       (384, C3D_FP64)])
def test_staged_xA_bit_identical(libc3d, n1m, prec):
    """xA's pieces with their rows staged in shared memory by bulk copies compute the same
    step bit for bit as with the rows read from global memory, for 2 and 8 rows per block."""
    g, dt = make_grid("small32", n1m=n1m, n2m=24, n3m=32)
    U, P, HH = ic.perturbed_laminar(g)
    out = []
    for xs, xw in ((0, 2), (1, 2), (1, 8)):
        ch = libc3d.Channel(g, prec)
        ch.upload(U, P, HH)
        s = ch.get_schedule()
        s.update(x_split_xA=1, x_stage_xA=xs, x_rows_per_block=xw)
        ch.set_schedule(s)
        for m in (1, 2, 3):
            ch.step(m, dt, 0.0, 0.0)
        out.append(ch.download())
        ch.close()
    for r in out[1:]:
        for a, b in zip(r, out[0]):
            assert np.array_equal(a, b)


def test_block_z_solve_mixed_close_to_segments(libc3d):
    """The block form of the z passes solves the cyclic systems exactly, the segment form to
    the FP32 warm-up tolerance: three mixed steps agree to FP32 rounding."""
    g, dt = make_grid("small32", n1m=64, n2m=48, n3m=384)
    U, P, HH = ic.perturbed_laminar(g)
    res = []
    for zl in (16, 0):
        ch = libc3d.Channel(g, C3D_MIXED)
        ch.upload(U, P, HH)
        s = ch.get_schedule()
        s.update({f"z_segment_z{c}": zl for c in "ABCDE"})
        ch.set_schedule(s)
        for m in (1, 2, 3):
            ch.step(m, dt, 0.0, 0.0)
        res.append(ch.download())
        ch.close()
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    for c, j0 in ((0, 1), (1, 2), (2, 1)):
        a = res[1][0][1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c]
        b = res[0][0][1:n1 + 1, j0:n2 + 1, 1:n3 + 1, c]
        assert rel(a, b) < 1e-5, (c, rel(a, b))


def test_stalled_stage_wait_becomes_error(libc3d):
    """The bounded wait of the bulk-copy stages runs out (on a barrier that nothing arrives
    on, with no copy in flight) and the flag it sets reaches the C-ABI as C3D_ECUDA."""
    g, dt = make_grid("tiny16")
    U, P, HH = ic.perturbed_laminar(g)
    ch = libc3d.Channel(g, C3D_MIXED)
    ch.upload(U, P, HH)
    ch.step(1, dt, 0.0, 0.0)
    L = libc3d.load()
    assert L.c3d_sync(ch.h) == 0
    assert L.c3d_pipe_wait_selftest(ch.h, 0.0) == -1          # limit out of range
    assert L.c3d_pipe_wait_selftest(ch.h, 5.0) == 0           # queued: waits 5 ms, then flags
    assert L.c3d_sync(ch.h) == -2
    assert b"bulk-copy stage" in L.c3d_last_error()
    with pytest.raises(libc3d.C3DError):
        ch.step(2, dt, 0.0, 0.0)
    ch.close()


@pytest.mark.parametrize("shape,prec", [((64, 48, 64), C3D_MIXED), ((96, 200, 32), C3D_MIXED), ((48, 24, 48), C3D_FP64),
                                        ((64, 130, 64), C3D_FP64)])
def test_ycn_tiles_bit_identical(libc3d, shape, prec):
    """The wall-normal CN factor with the planes staged in shared memory (tiles of 32 or 64
    columns, eight chunks of planes) performs the same recurrences as the register form:
    the step is bit-identical.  N2M = 200 and 130 give chunks of uneven length; 48 x 48
    columns leave a last tile of 32 columns for the 64-column tiles."""
    n1m, n2m, n3m = shape
    g, dt = make_grid("small32", n1m=n1m, n2m=n2m, n3m=n3m)
    U, P, HH = ic.perturbed_laminar(g)
    out = []
    for yt in (0, 32, 64):
        ch = libc3d.Channel(g, prec)
        ch.upload(U, P, HH)
        s = ch.get_schedule()
        s.update(ycn_tile=yt)
        ch.set_schedule(s)
        for m in (1, 2):
            ch.step(m, dt, 0.0, 0.0)
        out.append(ch.download())
        ch.close()
    for r in out[1:]:
        for a, b in zip(r, out[0]):
            assert np.array_equal(a, b)

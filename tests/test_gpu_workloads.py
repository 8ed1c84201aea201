"""GPU parity on the benchmark workloads themselves, against the FP64 CPU oracle.

The small-grid tests (test_gpu_parity.py, test_gpu_ops.py, test_gpu_les.py) pin the step
on grids up to 64^3; these repeat the comparison at the sizes the benchmark runs:

  * channel64 (64 x 65 x 64 points, 4pi x 2 x 4/3 pi, beta 2.0, RE 4200, dt 0.002):
    200 FP64 steps from the seeded perturbed-laminar start, relative L2 <= 1e-12 for
    u, v, w and HH and 1e-11 for P (measured: 1e-14 and 4e-13), PRESG to 1e-9 relative;
  * field256 (256 x 193 x 256 points): every operator of c3d_op_* in FP64 at 1e-13
    (1e-11 for GETDP), the mixed form's error at 2e-6 (2e-5 for GETDP);
  * channel384 (384 x 257 x 384 points, 2pi x 2 x pi, beta 2.2, RE 15000, dt 0.001):
    two FP64 steps after one oracle step, 1e-10 for u, v, w, HH and P, PRESG to 1e-7
    relative (GETUP forms DMPRESG as the difference of two sums of 3.8e7 O(1) terms
    divided by DT, so the oracle's own summation order moves it at the 1e-9 to 1e-8
    level; the CUDA path sums the increments UH - U, which has no cancellation); the
    mixed form after 20 steps from the same start, 1e-5 for u, v, w;
  * les128 (128 x 65 x 128 points, 8pi x 2 x 3pi, SGSCS + WALLMODEL_INSTANT): one FP64
    step after two oracle steps, 1e-10 for u, v, w, HH, P and SGSVIS, 1e-12 for the
    wall stresses.

The file runs last among the GPU parity tests because the oracle needs tens of seconds
per channel384 step; errors are printed (pytest -s) as well as asserted.
"""
import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, make_grid

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def interior(g, U, P, HH):
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    return dict(u=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0], v=U[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1],
                w=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2], p=P[:n1, :n2, :n3],
                hh=HH[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, :])


def errors(g, gpu, orc_fields):
    a, b = interior(g, *gpu), interior(g, *orc_fields)
    return {f: rel(a[f], b[f]) for f in a}


@pytest.fixture(scope="module")
def libc3d():
    from compact3d_gb300 import build, lib
    build.build()
    lib.load()
    return lib


def test_channel64_200_steps_fp64(libc3d, oracle_mod):
    g, dt = make_grid("channel64")
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    pg = pg3 = pgg = pg3g = 0.0
    worst = {}
    for n in range(1, 201):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
        pgg, pg3g = ch.step(n, dt, pgg, pg3g)
        if n in (1, 10, 50, 100, 200):
            e = errors(g, ch.download(), (U, P, HH))
            print(f"channel64 step {n}: " + " ".join(f"{k}={v:.2e}" for k, v in e.items()))
            for k, v in e.items():
                worst[k] = max(worst.get(k, 0.0), v)
    for f in ("u", "v", "w", "hh"):
        assert worst[f] < 1e-12, (f, worst[f])
    assert worst["p"] < 1e-11, worst["p"]
    assert pgg == pytest.approx(pg, rel=1e-9)


def operand(g, seed=11):
    U, _ = ic.band_limited(g, seed=seed)
    F = np.asfortranarray(U[..., 0])
    rng = np.random.default_rng(seed)
    F[1:g.n1m + 1, 0, 1:g.n3m + 1] = rng.normal(size=(g.n1m, g.n3m))
    F[1:g.n1m + 1, g.n2m + 1, 1:g.n3m + 1] = rng.normal(size=(g.n1m, g.n3m))
    return F


def test_field256_operators(libc3d, oracle_mod):
    g, _ = make_grid("field256")
    orc = oracle_mod.Oracle(g)
    c64 = libc3d.Channel(g, C3D_FP64)
    cmx = libc3d.Channel(g, C3D_MIXED)
    F = operand(g)
    for key, op in libc3d.OPS.items():
        j0 = 2 if op == libc3d.OPS["DY1"] else 1
        sl = (slice(1, g.n1m + 1), slice(j0, g.n2m + 1), slice(1, g.n3m + 1))
        Xo = orc.operator(op, F)[sl]
        e64 = rel(c64.operator(op, F)[sl], Xo)
        emx = rel(cmx.operator(op, F)[sl], Xo)
        print(f"field256 {key}: fp64 {e64:.2e} mixed {emx:.2e}")
        assert e64 < (1e-11 if key == "POISSON" else 1e-13), (key, e64)
        assert emx < (2e-5 if key == "POISSON" else 2e-6), (key, emx)
    c64.close()
    cmx.close()


@pytest.fixture(scope="module")
def channel384(oracle_mod):
    """Oracle trajectory of channel384 from the projected seeded start: the state after
    step 1 (the GPU runs start there, so HH_old and P are non-trivial), after step 3 and
    after step 21."""
    g, dt = make_grid("channel384")
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    pg = pg3 = 0.0
    snaps = {}
    for n in range(1, 22):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
        if n in (1, 3, 21):
            snaps[n] = (U.copy(order="F"), P.copy(order="F"), HH.copy(order="F"), pg, pg3)
    return g, dt, snaps


def test_channel384_two_steps_fp64(libc3d, channel384):
    g, dt, snaps = channel384
    U1, P1, H1, pg, pg3 = snaps[1]
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U1, P1, H1)
    for n in (2, 3):
        pg, pg3 = ch.step(n, dt, pg, pg3)
    e = errors(g, ch.download(), snaps[3][:3])
    ch.close()
    print("channel384 fp64 after 2 steps: " + " ".join(f"{k}={v:.2e}" for k, v in e.items()))
    for f in ("u", "v", "w", "hh", "p"):
        assert e[f] < 1e-10, (f, e[f])
    assert pg == pytest.approx(snaps[3][3], rel=1e-7)


def test_channel384_mixed_twenty_steps(libc3d, channel384):
    g, dt, snaps = channel384
    U1, P1, H1, pg, pg3 = snaps[1]
    ch = libc3d.Channel(g, C3D_MIXED)
    ch.upload(U1, P1, H1)
    for n in range(2, 22):
        pg, pg3 = ch.step(n, dt, pg, pg3)
    e = errors(g, ch.download(), snaps[21][:3])
    d = ch.diagnose()
    ch.close()
    print("channel384 mixed after 20 steps: " + " ".join(f"{k}={v:.2e}" for k, v in e.items())
          + f" divmax={d['divmax']:.2e}")
    for f in ("u", "v", "w"):
        assert e[f] < 1e-5, (f, e[f])
    assert e["p"] < 1e-4, e["p"]


def test_les128_one_step_fp64(libc3d, oracle_mod):
    g, dt = make_grid("les128")
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.loglaw(g, 2000.0, amp=0.05)
    orc.project(U)
    S = g.zeros_s()
    pg = pg3 = 0.0
    for n in (1, 2):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3, S)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    tw, tb, wsm = orc.get_wall()
    ch.upload_wall(tw, tb)
    ch.set_wsm(wsm)
    pgo, _ = orc.getup(U, P, HH, 3, dt, pg, pg3, S)
    pgg, _ = ch.step(3, dt, pg, pg3)
    e = errors(g, ch.download(), (U, P, HH))
    sl = (slice(1, g.n1m + 1), slice(0, g.n2m + 2), slice(1, g.n3m + 1))
    e["sgsvis"] = rel(ch.download_sgsvis()[sl], S[sl])
    tw, tb, wsm = orc.get_wall()
    twg, tbg = ch.download_wall()
    isl = (slice(1, g.n1m + 1), slice(1, g.n3m + 1), slice(None))
    e["tauw"], e["taub"] = rel(twg[isl], tw[isl]), rel(tbg[isl], tb[isl])
    e["wsm"] = abs(ch.get_wsm()[0] - wsm[0]) / abs(wsm[0])
    ch.close()
    print("les128 fp64 one step: " + " ".join(f"{k}={v:.2e}" for k, v in e.items()))
    for f in ("u", "v", "w", "hh", "p", "sgsvis"):
        assert e[f] < 1e-10, (f, e[f])
    for f in ("tauw", "taub", "wsm"):
        assert e[f] < 1e-12, (f, e[f])
    assert pgg == pytest.approx(pgo, rel=1e-9, abs=1e-15)

"""GPU parity of the wall-modelled LES step (FILES != 0) against the FP64 oracle: the SGS
models SGSDY, SGSCS and SGSSD with the wall models INSTANT, ROUGH, IWMLES (smooth and
rough), MARUSIC1, WERNER and PIOMELLI, and no-slip walls.

Tolerances (relative L2 over the interior unless stated):
  * FP64 form, one step: 1e-10 for U, V, W, HH, P and SGSVIS, 1e-12 for the
    wall stresses TAUW/TAUB and WSM(1) (the wall models are the same arithmetic).
  * IWMLES from NTIME = 1 over 12 steps: stresses 1e-8 (rough 1e-7) per step, the field
    1e-9 (its Newton Jacobian differences the residual over 1e-9 in u_tau).
  * FP64 form, 10 steps: 1e-9 for U, V, W.
  * mixed form against the FP64 GPU form after 20 steps: 1e-4 for U, V, W, 1e-3 for the
    mean wall stress (FP32 line solves and SGS fluxes; FP64 wall model and reductions).
The SGS fluxes are formed as three edge stresses instead of the reference's separate
terms (the sums are linear in the edge viscosity), which changes only rounding.
"""
import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, make_grid

pytestmark = pytest.mark.gpu

RETAU = 2000.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def interior(g, U, P, HH):
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    return dict(u=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0], v=U[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1],
                w=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2], p=P[:n1, :n2, :n3],
                hh=HH[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, :])


@pytest.fixture(scope="module")
def libc3d():
    from compact3d_gb300 import build, lib
    build.build()
    lib.load()
    return lib


def warm_start(oracle_mod, name, nwarm=2, **over):
    """Oracle state after `nwarm` LES steps from the projected log-law start (so WSM,
    the wall stresses and the AB2 history are all non-trivial)."""
    g, dt = make_grid(name, **over)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.loglaw(g, RETAU)
    orc.project(U)
    S = g.zeros_s()
    pg = pg3 = 0.0
    for n in range(1, nwarm + 1):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3, S)
    return g, dt, orc, U, P, HH, S, pg, pg3


def gpu_from(libc3d, orc, g, U, P, HH, precision=C3D_FP64):
    ch = libc3d.Channel(g, precision)
    ch.upload(U, P, HH)
    tw, tb, wsm = orc.get_wall()
    ch.upload_wall(tw, tb)
    ch.set_wsm(wsm)
    return ch


@pytest.mark.parametrize("name,over", [
    ("les32cs", {}),                        # Smagorinsky + WALLMODEL_INSTANT
    ("les32dy", {}),                        # dynamic + WALLMODEL_INSTANT
    ("les32cs", dict(wmodel=0, cks=2.0)),   # Smagorinsky, no-slip walls, stretched y
    ("les32dy", dict(wmodel=0, cks=2.0)),   # dynamic, no-slip walls, stretched y
    ("les32cs", dict(wmodel=4)),            # Smagorinsky + WALLMODEL_WERNER (both walls)
    ("les32dy", dict(wmodel=4)),            # dynamic + WALLMODEL_WERNER
    ("les32cs", dict(wmodel=3)),            # Smagorinsky + MARUSIC1, reference plane ZS = 1
    ("les32dy", dict(wmodel=3, n2m=32)),    # dynamic + MARUSIC1, ZS = 2
    ("les32cs", dict(wmodel=5)),            # Smagorinsky + PIOMELLI
    ("les32dy", dict(wmodel=5, y0=1e-5)),   # PIOMELLI with H(1) 5e-6 below YC(1): YP climbs
    ("les32dy", dict(files=3)),             # SGSSD (scale-dependent) + WALLMODEL_INSTANT
    ("les32dy", dict(files=3, wmodel=0, cks=2.0)),   # SGSSD, no-slip walls, stretched y
    ("les32dy", dict(files=3, wmodel=3)),   # SGSSD + MARUSIC1
    ("les32cs", dict(y0=2e-3)),             # Smagorinsky + WALLMODEL_ROUGH (Y0 != 0)
])
def test_les_one_step_fp64(libc3d, oracle_mod, name, over):
    g, dt, orc, U, P, HH, S, pg, pg3 = warm_start(oracle_mod, name, **over)
    ch = gpu_from(libc3d, orc, g, U, P, HH)
    n = 3
    pgo, pg3o = orc.getup(U, P, HH, n, dt, pg, pg3, S)
    pgg, pg3g = ch.step(n, dt, pg, pg3)
    Ug, Pg, Hg = ch.download()
    a, b = interior(g, Ug, Pg, Hg), interior(g, U, P, HH)
    for f in ("u", "v", "w", "hh"):
        assert rel(a[f], b[f]) < 1e-10, (f, rel(a[f], b[f]))
    assert rel(a["p"], b["p"]) < 1e-10, rel(a["p"], b["p"])
    Sg = ch.download_sgsvis()
    sl = (slice(1, g.n1m + 1), slice(0, g.n2m + 2), slice(1, g.n3m + 1))
    assert np.abs(S[sl]).max() > 0
    assert rel(Sg[sl], S[sl]) < 1e-10, rel(Sg[sl], S[sl])
    assert pgg == pytest.approx(pgo, rel=1e-9, abs=1e-15)
    tw, tb, wsm = orc.get_wall()
    twg, tbg = ch.download_wall()
    isl = (slice(1, g.n1m + 1), slice(1, g.n3m + 1), slice(None))
    if g.wmodel:
        assert rel(twg[isl], tw[isl]) < 1e-12 and rel(tbg[isl], tb[isl]) < 1e-12
        assert ch.get_wsm()[0] == pytest.approx(wsm[0], rel=1e-12)
    else:
        np.testing.assert_allclose(ch.get_wsm(), wsm, rtol=1e-10, atol=1e-18)


def test_les_ten_steps_fp64(libc3d, oracle_mod):
    g, dt, orc, U, P, HH, S, pg, pg3 = warm_start(oracle_mod, "les32cs")
    ch = gpu_from(libc3d, orc, g, U, P, HH)
    pgg, pg3g = pg, pg3
    for n in range(3, 13):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3, S)
        pgg, pg3g = ch.step(n, dt, pgg, pg3g)
    Ug, Pg, Hg = ch.download()
    a, b = interior(g, Ug, Pg, Hg), interior(g, U, P, HH)
    for f in ("u", "v", "w"):
        assert rel(a[f], b[f]) < 1e-9, (f, rel(a[f], b[f]))
    d = ch.diagnose()
    assert d["divmax"] < 1e-12


@pytest.mark.parametrize("name,over", [("les32dy", {}), ("les32cs", dict(wmodel=3)), ("les32dy", dict(wmodel=5)),
                                       ("les32dy", dict(files=3))])
def test_les_mixed_against_fp64(libc3d, oracle_mod, name, over):
    g, dt, orc, U, P, HH, S, pg, pg3 = warm_start(oracle_mod, name, **over)
    c64 = gpu_from(libc3d, orc, g, U, P, HH, C3D_FP64)
    cmx = gpu_from(libc3d, orc, g, U, P, HH, C3D_MIXED)
    for c in (c64, cmx):
        c.set_presg(pg, pg3)
    for n in range(3, 23):
        c64.step_async(n, dt)
        cmx.step_async(n, dt)
    a = interior(g, *cmx.download())
    b = interior(g, *c64.download())
    for f in ("u", "v", "w"):
        assert rel(a[f], b[f]) < 1e-4, (f, rel(a[f], b[f]))
    w64, wmx = c64.get_wsm()[0], cmx.get_wsm()[0]
    assert wmx == pytest.approx(w64, rel=1e-3)
    assert cmx.diagnose()["divmax"] < 1e-3


def test_les_wall_model_iteration_cap(libc3d, oracle_mod):
    """A cap of 2 Newton iterations cannot converge: the step completes, reports
    C3D_ENOTCONV, and the channel stays usable (the next step with the default cap
    succeeds)."""
    g, dt, orc, U, P, HH, S, pg, pg3 = warm_start(oracle_mod, "les32cs", nwarm=1)
    ch = gpu_from(libc3d, orc, g, U, P, HH)
    ch.set_wall_iter_cap(2)
    with pytest.raises(libc3d.C3DError) as e:
        ch.step(2, dt, pg, pg3)
    assert e.value.code == -4
    ch.set_wall_iter_cap(10000)
    ch.step(3, dt, pg, pg3)
    Ug, _, _ = ch.download()
    assert np.isfinite(Ug).all()


@pytest.mark.parametrize("name,over,tol", [("les32cs", dict(wmodel=2), 1e-8), ("les32dy", dict(wmodel=2, n2m=64), 1e-8),
                                           ("les32cs", dict(wmodel=2, y0=1e-3), 1e-7)])
def test_iwmles_steps_fp64(libc3d, oracle_mod, name, over, tol):
    """WALLMODEL_IWMLES_SMOOTH / _ROUGH (WMODEL 2) from NTIME = 1 on both sides for 12 steps
    (two model updates): wall stresses and WSM(1) within 1e-8 (rough: 1e-7, its stress is a
    product of three Newton-derived factors) after every step (the Newton Jacobian
    differences the residual over 1e-9, which amplifies last-bit differences of pow and
    log), the field within 1e-9 at the end."""
    g, dt = make_grid(name, **over)
    orc = oracle_mod.Oracle(g)
    orc.set_cflmax(0.5)
    U, P, HH = ic.loglaw(g, RETAU)
    orc.project(U)
    S = g.zeros_s()
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    ch.set_cflmax(0.5)
    pg = pg3 = pgg = pg3g = 0.0
    isl = (slice(1, g.n1m + 1), slice(1, g.n3m + 1), 0)
    for n in range(1, 13):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3, S)
        pgg, pg3g = ch.step(n, dt, pgg, pg3g)
        tw, tb, wsm = orc.get_wall()
        twg, tbg = ch.download_wall()
        scale = max(np.abs(tw[isl]).max(), 1e-300)
        assert np.abs(twg[isl] - tw[isl]).max() <= tol * scale, n
        assert np.abs(tbg[isl] - tb[isl]).max() <= tol * max(scale, np.abs(tb[isl]).max()), n
        assert ch.get_wsm()[0] == pytest.approx(wsm[0], rel=tol, abs=1e-300), n
    Ug, Pg, Hg = ch.download()
    a, b = interior(g, Ug, Pg, Hg), interior(g, U, P, HH)
    for f in ("u", "v", "w"):
        assert rel(a[f], b[f]) < 1e-9, (f, rel(a[f], b[f]))

"""GPU parity: the CUDA step through the C-ABI against the FP64 CPU oracle.

Tolerances (relative L2 over the interior of each field unless stated):
  * FP64 form, one step:          1e-10 for U, V, W, HH and P; PRESG to 1e-9 relative.
  * FP64 form, 20 steps:          1e-9 for U, V, W.
  * mixed form (FP32 line solves, RHS and FFT; FP64 state, reductions and Poisson
    tridiagonal solves): 2e-5 relative L2 for U, V, W after 20 steps.
"""
import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, make_grid

pytestmark = pytest.mark.gpu


def interior(g, U, P, HH):
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    u = U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0]
    v = U[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1]
    w = U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2]
    p = P[:n1, :n2, :n3]
    h = HH[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, :]
    return dict(u=u, v=v, w=w, p=p, hh=h)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def libc3d():
    from compact3d_gb300 import build, lib
    build.build()
    lib.load()
    return lib


def start(oracle_mod, name, **over):
    g, dt = make_grid(name, **over)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    return g, dt, orc, U, P, HH


@pytest.mark.parametrize("name", ["tiny16", "small32", "channel64"])
def test_fp64_one_step(libc3d, oracle_mod, name):
    g, dt, orc, U, P, HH = start(oracle_mod, name)
    # give the AB2 history a non-zero HH_old and the pressure a non-zero field
    pg = pg3 = 0.0
    pg, pg3 = orc.getup(U, P, HH, 1, dt, pg, pg3)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    Ug, Pg, Hg = U.copy(order="F"), P.copy(order="F"), HH.copy(order="F")
    pgo, pg3o = orc.getup(U, P, HH, 2, dt, pg, pg3)
    pgg, pg3g = ch.step(2, dt, pg, pg3)
    Ug, Pg, Hg = ch.download(Ug, Pg, Hg)
    a, b = interior(g, Ug, Pg, Hg), interior(g, U, P, HH)
    for f in ("u", "v", "w", "hh"):
        assert rel(a[f], b[f]) < 1e-10, (f, rel(a[f], b[f]))
    assert rel(a["p"], b["p"]) < 1e-10, rel(a["p"], b["p"])
    assert pgg == pytest.approx(pgo, rel=1e-9, abs=1e-15)
    assert pg3g == pytest.approx(pg3o, abs=1e-12)


def test_fp64_twenty_steps(libc3d, oracle_mod):
    g, dt, orc, U, P, HH = start(oracle_mod, "small32")
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    pg = pg3 = 0.0
    pgg = pg3g = 0.0
    for n in range(1, 21):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
        pgg, pg3g = ch.step(n, dt, pgg, pg3g)
    Ug, Pg, Hg = ch.download()
    a, b = interior(g, Ug, Pg, Hg), interior(g, U, P, HH)
    for f in ("u", "v", "w"):
        assert rel(a[f], b[f]) < 1e-9, (f, rel(a[f], b[f]))
    assert pgg == pytest.approx(pg, rel=1e-8)


def test_diagnostics_match_oracle(libc3d, oracle_mod):
    g, dt, orc, U, P, HH = start(oracle_mod, "small32")
    pg = pg3 = 0.0
    for n in range(1, 4):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    d = ch.diagnose()
    o = orc.diagnose(U)
    assert d["cflm"] == pytest.approx(o["cflm"], rel=1e-12)
    assert d["flow1"] == pytest.approx(o["flow1"], rel=1e-12)
    assert d["flow3"] == pytest.approx(o["flow3"], abs=1e-12)
    assert np.allclose(d["wsm"], o["wsm"], rtol=1e-11)
    assert d["divmax"] < 1e-11 and o["divmax"] < 1e-11
    assert not d["nonfinite"]


def test_projection_matches_oracle(libc3d, oracle_mod):
    g, _ = make_grid("small32")
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    ch.project()
    orc.project(U)
    Ug, _, _ = ch.download()
    a, b = interior(g, Ug, P, HH), interior(g, U, P, HH)
    for f in ("u", "v", "w"):
        assert rel(a[f], b[f]) < 1e-12, f
    assert ch.diagnose()["divmax"] < 1e-12


def test_getup_host_arrays(libc3d, oracle_mod):
    """c3d_getup (upload, step, download per call) equals the device-resident path."""
    g, dt, orc, U, P, HH = start(oracle_mod, "tiny16")
    ch1 = libc3d.Channel(g, C3D_FP64)
    ch2 = libc3d.Channel(g, C3D_FP64)
    ch2.upload(U, P, HH)
    U1, P1, H1 = U.copy(order="F"), P.copy(order="F"), HH.copy(order="F")
    a = b = 0.0
    c = d = 0.0
    for n in range(1, 4):
        a, b = ch1.getup(U1, P1, H1, n, dt, a, b)
        c, d = ch2.step(n, dt, c, d)
    U2, P2, H2 = ch2.download()
    x, y = interior(g, U1, P1, H1), interior(g, U2, P2, H2)
    for f in ("u", "v", "w", "p", "hh"):
        assert np.array_equal(x[f], y[f]), f
    assert a == c and b == d


def test_mixed_error_bound(libc3d, oracle_mod):
    g, dt, orc, U, P, HH = start(oracle_mod, "small32")
    ch = libc3d.Channel(g, C3D_MIXED)
    ch.upload(U, P, HH)
    pg = pg3 = 0.0
    pgg = pg3g = 0.0
    for n in range(1, 21):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
        pgg, pg3g = ch.step(n, dt, pgg, pg3g)
    Ug, Pg, Hg = ch.download()
    a, b = interior(g, Ug, Pg, Hg), interior(g, U, P, HH)
    for f in ("u", "v", "w"):
        assert rel(a[f], b[f]) < 2e-5, (f, rel(a[f], b[f]))
    d = ch.diagnose()
    assert d["divmax"] < 1e-3
    assert d["flow1"] == pytest.approx(orc.chkmf(U)[0], rel=1e-9)


def test_bad_dt_rejected(libc3d, oracle_mod):
    g, dt, orc, U, P, HH = start(oracle_mod, "tiny16")
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    with pytest.raises(libc3d.C3DError):
        ch.step(1, -1.0, 0.0, 0.0)
    with pytest.raises(libc3d.C3DError):
        ch.step(1, float("nan"), 0.0, 0.0)


def test_nonfinite_detected(libc3d, oracle_mod):
    g, dt, orc, U, P, HH = start(oracle_mod, "tiny16")
    U[3, 4, 5, 0] = np.nan
    ch = libc3d.Channel(g, C3D_FP64)
    ch.upload(U, P, HH)
    assert ch.diagnose()["nonfinite"]

"""The oracle restatement pinned against the reference's own routines (CPU only).

compact3d.f is translated to C by oracle/f77c.py and compiled with gcc (oracle/ref.py):
its GETUP, MESH, INDICES, INIWAVE/METRICPOISSON, DIVCHECK, CFL, CHKMF, WALLSS and every
SGS and wall model run unchanged, with FFTW replaced by the DFT it documents
(oracle/fftw_shim.c).  These tests compare the oracle with them on the same inputs, and
both with the committed golden fixtures (tests/golden/, made by make_golden.py from the
translated reference).

Tolerances (relative L2 over the interior unless stated; both sides FP64):
  * MESH metrics and the Poisson tables (modified wavenumbers, y stencil): exact;
  * DIVCHECK, CFL, CHKMF, WALLSS: 1e-14;
  * GETUP, five steps: 1e-13 for u, v, w, HH and SGSVIS, 1e-10 for P (the pinned mean
    pressure mode of GETDP is a near-singular solve, and the oracle's FFT and FFTW's
    transform order differ), 1e-12 for the wall stresses; PRESG to 1e-8 relative (it is
    the difference of two sums of O(1) terms over the whole channel, divided by DT, so
    the summation order of the OpenMP reductions moves it at that level);
  * WALLMODEL_IWMLES_ROUGH: 1e-7, because its Newton solve uses a finite-difference
    Jacobian with a 1e-9 step that turns last-bit differences into different iterates,
    which agree only to the iteration's tolerance.
Skipped where neither the reference source nor an earlier translation is present.
"""
import os

import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import make_grid, mesh

ref = pytest.importorskip("oracle.ref")
pytestmark = pytest.mark.skipif(not ref.available(), reason="reference source not present")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def interior(g, U, P, HH):
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    return dict(u=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0], v=U[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1],
                w=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2], p=P[:n1, :n2, :n3], hh=HH[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, :])


@pytest.mark.parametrize("n,alx,aly,alz,wmodel,y0", [
    ((17, 17, 17), 6.0, 2.0, 3.0, 0, 0.0),      # full channel, tanh grid
    ((33, 25, 49), 6.0, 1.0, 3.0, 0, 0.0),      # half channel (free-slip top), tanh grid
    ((33, 17, 33), 25.0, 2.0, 9.0, 1, 0.0),     # wall model: uniform y
    ((33, 17, 33), 25.0, 2.0, 9.0, 1, 2e-3),    # rough wall: uniform y from Y0
])
def test_mesh_matches_reference(n, alx, aly, alz, wmodel, y0):
    """compact3d_gb300.grid.mesh restates MESH (compact3d.f:302-443); with the reference's
    hard-coded CKS = 2.5 the two give the same metrics bit for bit."""
    from compact3d_gb300.grid import Grid
    g = Grid(n1m=n[0] - 1, n2m=n[1] - 1, n3m=n[2] - 1, alx=alx, aly=aly, alz=alz, re=1000.0, cks=2.5,
             wmodel=wmodel, y0=y0)
    R = ref.RefChannel(g, reference_mesh=True)
    a = mesh(*n, alx, aly, alz, 2.5, wmodel, y0)
    b = R.mesh()
    for k in ("y", "dy", "h", "hm", "hc", "hp", "dym", "dyc", "dyp"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for k in ("aly", "vol", "dx1", "dx3"):
        assert a[k] == b[k], k


@pytest.mark.parametrize("name", ["tiny16", "small32"])
def test_poisson_tables_match_reference(oracle_mod, name):
    """INIWAVE's modified wavenumbers and METRICPOISSON's stencil (compact3d.f:9182-9263)."""
    g, _ = make_grid(name)
    R = ref.RefChannel(g)
    o = dict(zip(("ak1", "ak3", "pmj", "pcj", "ppj"), oracle_mod.Oracle(g).poisson_metrics()))
    r = R.poisson_metrics()
    for k in ("ak1", "ak3", "pmj", "pcj", "ppj"):
        np.testing.assert_array_equal(o[k], r[k], err_msg=k)


@pytest.mark.parametrize("name", ["tiny16", "small32"])
def test_getup_matches_reference(oracle_mod, name):
    g, dt = make_grid(name)
    orc = oracle_mod.Oracle(g)
    R = ref.RefChannel(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    U2, P2, H2 = U.copy(order="F"), P.copy(order="F"), HH.copy(order="F")
    pg = pg3 = qg = qg3 = 0.0
    for n in range(1, 6):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
        qg, qg3 = R.getup(U2, P2, H2, n, dt, qg, qg3)
        a, b = interior(g, U, P, HH), interior(g, U2, P2, H2)
        for f in ("u", "v", "w", "hh"):
            assert rel(a[f], b[f]) < 1e-13, (n, f, rel(a[f], b[f]))
        assert rel(a["p"], b["p"]) < 1e-10, (n, rel(a["p"], b["p"]))
        assert pg == pytest.approx(qg, rel=1e-8)
        assert pg3 == pytest.approx(qg3, rel=1e-8, abs=1e-15)
    assert orc.divcheck(U) == pytest.approx(R.divcheck(U), rel=1e-14, abs=1e-18)
    assert orc.cfl(U) == pytest.approx(R.cfl(U), rel=1e-14)
    f1, f3 = orc.chkmf(U)
    r1, r3 = R.chkmf(U)
    assert f1 == pytest.approx(r1, rel=1e-14) and f3 == pytest.approx(r3, rel=1e-10, abs=1e-17)
    np.testing.assert_allclose(orc.wallss(U), R.wallss(U, P), rtol=1e-14, atol=1e-20)


LES_CASES = [
    ("les32cs", {}),                        # SGSCS + WALLMODEL_INSTANT
    ("les32dy", {}),                        # SGSDY + WALLMODEL_INSTANT
    ("les32cs", dict(wmodel=0, cks=2.0)),   # SGSCS, no-slip walls (WALLSS before GETUP)
    ("les32dy", dict(wmodel=0, cks=2.0)),   # SGSDY, no-slip walls
    ("les32cs", dict(wmodel=4)),            # WALLMODEL_WERNER
    ("les32cs", dict(wmodel=3)),            # WALLMODEL_MARUSIC1
    ("les32cs", dict(wmodel=5)),            # WALLMODEL_PIOMELLI
    ("les32dy", dict(files=3)),             # SGSSD + WALLMODEL_INSTANT
    ("les32dy", dict(files=3, wmodel=0, cks=2.0)),   # SGSSD, no-slip walls
    ("les32cs", dict(y0=2e-3)),             # WALLMODEL_ROUGH
    ("les32cs", dict(wmodel=2)),            # WALLMODEL_IWMLES_SMOOTH (update at step 5 and 10)
    ("les32cs", dict(wmodel=2, y0=2e-3)),   # WALLMODEL_IWMLES_ROUGH
]


@pytest.mark.parametrize("name,over", LES_CASES)
def test_les_matches_reference(oracle_mod, name, over):
    g, dt = make_grid(name, **over)
    orc = oracle_mod.Oracle(g)
    R = ref.RefChannel(g)
    U, P, HH = ic.loglaw(g, 2000.0)
    orc.project(U)
    U2, P2, H2 = U.copy(order="F"), P.copy(order="F"), HH.copy(order="F")
    S, S2 = g.zeros_s(), g.zeros_s()
    tw, tb, wsm = orc.get_wall()
    R.set_wall(tw, tb)
    R.set_wsm(wsm)
    rough_iwm = g.wmodel == 2 and g.y0 != 0.0
    tol = 1e-7 if rough_iwm else 1e-13
    tolw = 1e-7 if rough_iwm else 1e-12
    pg = pg3 = qg = qg3 = 0.0
    n1, n3 = g.n1m, g.n3m
    for n in range(1, (11 if g.wmodel == 2 else 3) + 1):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3, S)
        qg, qg3 = R.getup(U2, P2, H2, n, dt, qg, qg3, S2)
        a, b = interior(g, U, P, HH), interior(g, U2, P2, H2)
        for f in ("u", "v", "w", "hh"):
            assert rel(a[f], b[f]) < tol, (n, f, rel(a[f], b[f]))
        assert rel(a["p"], b["p"]) < (1e-6 if rough_iwm else 1e-10), (n, rel(a["p"], b["p"]))
        sl = (slice(1, n1 + 1), slice(None), slice(1, n3 + 1))
        assert rel(S[sl], S2[sl]) < (1e-7 if rough_iwm else 1e-11), (n, rel(S[sl], S2[sl]))
        w1, b1, m1 = orc.get_wall()
        w2, b2, m2 = R.get_wall()
        isl = (slice(1, n1 + 1), slice(1, n3 + 1))
        assert rel(w1[isl], w2[isl]) < tolw and rel(b1[isl], b2[isl]) < tolw, n
        assert m1[0] == pytest.approx(m2[0], rel=tolw, abs=1e-300)


def test_golden_fixtures_match_oracle(oracle_mod):
    """The oracle against the committed fixtures of the reference's GETUP (DNS and LES)."""
    for fname, name, over, les in (("tiny16_dns.npz", "tiny16", {}, False),
                                   ("les16_les.npz", "les32cs", dict(n1m=16, n3m=16), True)):
        d = np.load(os.path.join(GOLDEN, fname))
        g, dt = make_grid(name, **over)
        orc = oracle_mod.Oracle(g)
        U, P, HH = (np.asfortranarray(d[k]) for k in ("U0", "P0", "HH0"))
        S = g.zeros_s() if les else None
        if les:
            orc.set_wall(np.asfortranarray(d["TAUW0"]), np.asfortranarray(d["TAUB0"]))
            orc.set_wsm(d["WSM0"])
        pg = pg3 = 0.0
        for n in range(1, int(d["steps"]) + 1):
            pg, pg3 = orc.getup(U, P, HH, n, float(d["dt"]), pg, pg3, S)
            assert pg == pytest.approx(d["PRESG"][n - 1, 0], rel=1e-8)
        a, b = interior(g, U, P, HH), interior(g, d["U"], d["P"], d["HH"])
        for f in ("u", "v", "w", "hh"):
            assert rel(a[f], b[f]) < 1e-13, (fname, f, rel(a[f], b[f]))
        assert rel(a["p"], b["p"]) < 1e-10, (fname, rel(a["p"], b["p"]))
        # max|div u| is at the rounding level of the state (1e-16 of |u|)
        assert orc.divcheck(U) == pytest.approx(float(d["DIVMAX"]), abs=1e-14)
        assert orc.cfl(U) == pytest.approx(float(d["CFLM"]), rel=1e-14)
        if les:
            tw, tb, wsm = orc.get_wall()
            assert rel(tw, d["TAUW"]) < 1e-12 and rel(tb, d["TAUB"]) < 1e-12
            sl = (slice(1, g.n1m + 1), slice(None), slice(1, g.n3m + 1))
            assert rel(S[sl], d["SGSVIS"][sl]) < 1e-12


@pytest.mark.parametrize("name", ["tiny16", "small32"])
def test_openmp_translation_matches_serial(name):
    """The reference with its !$OMP PARALLEL DO loops kept (the form the benchmark's
    reference arm times) computes the serial translation's steps to rounding: five steps,
    1e-13 for u, v, w, HH, 1e-10 for P (only the order of the OpenMP reductions differs)."""
    g, dt = make_grid(name)
    A = ref.RefChannel(g)
    B = ref.RefChannel(g, omp=True)
    U, P, HH = ic.perturbed_laminar(g)
    X = [x.copy(order="F") for x in (U, P, HH)]
    Y = [x.copy(order="F") for x in (U, P, HH)]
    pa = pa3 = pb = pb3 = 0.0
    for n in range(1, 6):
        pa, pa3 = A.getup(*X, n, dt, pa, pa3)
        pb, pb3 = B.getup(*Y, n, dt, pb, pb3)
    a, b = interior(g, *X), interior(g, *Y)
    for f in ("u", "v", "w", "hh"):
        assert rel(b[f], a[f]) < 1e-13, (f, rel(b[f], a[f]))
    assert rel(b["p"], a["p"]) < 1e-10
    assert pb == pytest.approx(pa, rel=1e-8)

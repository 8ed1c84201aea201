"""Known-answer tests of the oracle's LES restatement (CPU only).

The reference ships no tests for its SGS models or wall model, so the restatement of
STRAIN (compact3d.f:5558-5689), SGSCS (1413-1488), SGSDY (1250-1400), FILTER
(5190-5228), WALLMODEL_INSTANT (2319-2493) and the SGS fluxes of RHS1-3 is pinned by
closed forms: linear shear, the law of the wall, invariances of the dynamic procedure and
the modified wavenumbers of the compact operators for a constant eddy viscosity.
"""
import math

import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import make_grid


def _grid(name="les32cs", **over):
    g, dt = make_grid(name, **over)
    return g, dt


def _xc(g):
    return (np.arange(g.n1m) + 0.5) * g.alx / g.n1m


def _xf(g):
    return np.arange(g.n1m) * g.alx / g.n1m


def _zf(g):
    return np.arange(g.n3m) * g.alz / g.n3m


def _yc(g):
    Y = g.arrays["y"]
    return 0.5 * (Y[1:g.n2m + 1] + Y[2:g.n2m + 2])


def _ak(n, dxinv, m):
    """(1,22,1) compact first derivative applied twice: modified wavenumber squared."""
    th = 2 * math.pi * m / n
    return 288.0 * dxinv ** 2 * (1 - math.cos(th)) / (11 + math.cos(th)) ** 2


def test_sgscs_linear_shear_closed_form(oracle_mod):
    """u = a*y (cell centres), v = w = 0: S12 = a/2 everywhere (the wall-model branch of
    STRAIN included), |S| = a, and SGSCS gives C_s(J)^2 DXYZ^(2/3) a with the Van Driest
    damping of y+ = (Y(J)+DY(J)/2) u_tau RE, u_tau = (WSM1^2+WSM3^2)^(1/4)."""
    g, _ = _grid("les32cs")
    o = oracle_mod.Oracle(g)
    a = 0.37
    U = g.zeros_u()
    U[1:g.n1m + 1, 1:g.n2m + 1, 1:g.n3m + 1, 0] = a * _yc(g)[None, :, None]
    wsm = np.array([4.1e-4, 0.0, 1.3e-4])
    o.set_wsm(wsm)
    S, smagc = o.sgs(U)
    utau = math.sqrt(math.sqrt(wsm[0] ** 2 + wsm[2] ** 2))
    Y, DY = g.arrays["y"], g.arrays["dy"]
    for J in range(1, g.n2m + 1):
        yp = (Y[J] + DY[J] * 0.5) * utau * g.re
        cs = 0.1 * (1 - math.exp(-yp / 26.0))
        assert smagc[J - 1] == pytest.approx(cs * cs, rel=1e-14)
        dxyz = 1.0 / g.arrays["dx1"] * DY[J] / g.arrays["dx3"]
        want = max(cs * cs * dxyz ** (2.0 / 3.0) * a, -1.0 / g.re)
        got = S[1:g.n1m + 1, J, 1:g.n3m + 1]
        np.testing.assert_allclose(got, want, rtol=1e-12)
    # wall planes untouched (zero)
    assert np.all(S[:, 0, :] == 0) and np.all(S[:, g.n2m + 1, :] == 0)


def _smooth_field(g, seed=3):
    U, P, HH = ic.loglaw(g, 2000.0, amp=0.2, seed=seed)
    return U


def test_sgsdy_galilean_and_scaling(oracle_mod):
    """The dynamic coefficient is invariant to a uniform velocity shift (strain and
    Leonard stress are differences) and to scaling of the field; the viscosity scales
    with |S| where the clipping at -1/RE is inactive."""
    g, _ = _grid("les32dy")
    o = oracle_mod.Oracle(g)
    U = _smooth_field(g)
    S0, c0 = o.sgs(U)
    U1 = U.copy(order="F")
    U1[..., 0] += 0.3
    U1[..., 2] -= 0.2
    S1, c1 = o.sgs(U1)
    np.testing.assert_allclose(c1, c0, rtol=1e-7, atol=1e-12)
    U2 = (2.0 * U).copy(order="F")
    S2, c2 = o.sgs(U2)
    np.testing.assert_allclose(c2, c0, rtol=1e-10, atol=1e-14)
    live = (S0 > -0.25 / g.re)
    np.testing.assert_allclose(S2[live], 2.0 * S0[live], rtol=1e-10, atol=1e-18)
    assert np.isfinite(S0).all() and np.any(S0 != 0)


def test_sgsdy_shift_invariance(oracle_mod):
    """FILTER and the plane sums of SGSDY commute with a periodic shift: moving the
    field by one cell in x leaves every plane's dynamic coefficient unchanged."""
    g, _ = _grid("les32dy")
    o = oracle_mod.Oracle(g)
    U = _smooth_field(g, seed=5)
    S0, c0 = o.sgs(U)
    Us = np.roll(U, 1, axis=0)
    Us[0] = U[0]
    Us[g.n1m + 1] = U[g.n1m + 1]
    Us[1:g.n1m + 1] = np.roll(U[1:g.n1m + 1], 1, axis=0)
    S1, c1 = o.sgs(np.asfortranarray(Us))
    np.testing.assert_allclose(c1, c0, rtol=1e-10, atol=1e-14)


def test_wallmodel_recovers_log_law(oracle_mod):
    """u(I,3,K), w(I,3,K) on the log law for a known u_tau: TAUW1 = u_tau^2 (to the
    Newton tolerance 1e-6 on u_tau), split along the velocity direction; WSM(1) is the
    plane mean."""
    g, _ = _grid("les32cs")
    o = oracle_mod.Oracle(g)
    DY = g.arrays["dy"]
    deltap = DY[1] + DY[2] + DY[3] / 2.0
    rng = np.random.default_rng(7)
    ut = rng.uniform(0.01, 0.05, size=(g.n1m, g.n3m))
    mag = ut * (np.log(ut * deltap * g.re) / 0.41 + 5.2)
    ang = rng.uniform(-0.4, 0.4, size=(g.n1m, g.n3m))
    U = g.zeros_u()
    U[1:g.n1m + 1, 3, 1:g.n3m + 1, 0] = mag * np.cos(ang)
    U[1:g.n1m + 1, 3, 1:g.n3m + 1, 2] = mag * np.sin(ang)
    assert o.wallmodel(U) == 0
    tw, tb, wsm = o.get_wall()
    tau = np.hypot(tw[1:g.n1m + 1, 1:g.n3m + 1, 0], tb[1:g.n1m + 1, 1:g.n3m + 1, 0])
    np.testing.assert_allclose(tau, ut ** 2, rtol=2e-4)
    np.testing.assert_allclose(np.arctan2(tb[1:g.n1m + 1, 1:g.n3m + 1, 0], tw[1:g.n1m + 1, 1:g.n3m + 1, 0]),
                               ang, atol=1e-12)
    assert wsm[0] == pytest.approx(tau.mean(), rel=1e-12)
    # the top-wall stresses are not modelled
    assert np.all(tw[..., 1] == 0) and np.all(tb[..., 1] == 0)


WW = dict(B=0.1428571429, AB1=7.202125274, AB3=69.74057973, AB4=0.1376936317, AB5=1.75)


def _werner_tau(vel, dy, re, wsm1):
    """Werner-Wengle stress magnitude at the first cell centre (compact3d.f:4855-4869)."""
    vcase = WW["AB3"] * np.sqrt(abs(wsm1)) / 11.81
    visc = 2.0 * vel / dy / re
    power = (WW["AB1"] * (1.0 / dy / re) ** (1.0 + WW["B"]) + WW["AB4"] * (1.0 / dy / re) ** WW["B"] * vel) ** WW["AB5"]
    return np.where(vel <= vcase, visc, power)


@pytest.mark.parametrize("wsm1", [1e-6, 10.0])   # power-law branch, viscous branch
def test_werner_matches_numpy_restatement(oracle_mod, wsm1):
    """WALLMODEL_WERNER on a random field against an independent numpy restatement with
    the reference's indexing (x neighbour IPA(K)/IMA(K) taken with the z index, F:4852,
    4881, 4924), both walls, both branches of the power law; WSM(1) is the plane mean of
    the bottom u-stress at the cell centres and WSM(2), WSM(3) are zeroed."""
    g, _ = _grid("les32cs", wmodel=4)
    o = oracle_mod.Oracle(g)
    U = _smooth_field(g, seed=11)
    o.set_wsm([wsm1, 0.3, 0.4])
    assert o.wallmodel(U) == 0
    tw, tb, wsm = o.get_wall()
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    DY = g.arrays["dy"]
    i = np.arange(1, n1 + 1)[:, None]
    k = np.arange(1, n3 + 1)[None, :]
    ipa = lambda q: np.where(q == n1, 1, q + 1)
    ima = lambda q: np.where(q == 1, n1, q - 1)
    kpa = lambda q: np.where(q == n3, 1, q + 1)
    kma = lambda q: np.where(q == 1, n3, q - 1)
    te = []
    for jw in (1, n2):
        u1 = 0.5 * (U[i, jw, k, 0] + U[ipa(k) + 0 * i, jw, k, 0])
        u2 = 0.5 * (U[i, jw, k, 2] + U[i, jw, kpa(k), 2])
        vel = np.sqrt(u1 ** 2 + u2 ** 2)
        t = _werner_tau(vel, DY[jw], g.re, wsm1)
        te.append((t * u1 / vel, t * u2 / vel))
    for wall, (tu, tw_) in enumerate(te):
        full_u = np.zeros((n1 + 1, n3 + 1)); full_u[1:, 1:] = tu
        full_w = np.zeros((n1 + 1, n3 + 1)); full_w[1:, 1:] = tw_
        exp_tw = 0.5 * (full_u[i, k] + full_u[ima(k) + 0 * i, k])
        exp_tb = 0.5 * (full_w[i, k] + full_w[i, kma(k)])
        np.testing.assert_allclose(tw[1:n1 + 1, 1:n3 + 1, wall], exp_tw, rtol=1e-12)
        np.testing.assert_allclose(tb[1:n1 + 1, 1:n3 + 1, wall], exp_tb, rtol=1e-12, atol=1e-18)
    assert wsm[0] == pytest.approx(te[0][0].mean(), rel=1e-12)
    assert wsm[1] == 0.0 and wsm[2] == 0.0


def test_werner_needs_n3_le_n1(oracle_mod):
    """The reference's IPA(K) indexing reads past the x index arrays when N3M > N1M; the
    restatement refuses such grids."""
    g, dt = _grid("les32cs", wmodel=4, n3m=64)
    o = oracle_mod.Oracle(g)
    U, P, HH = ic.loglaw(g, 2000.0)
    with pytest.raises(Exception):
        o.getup(U, P, HH, 1, dt, 0.0, 0.0, g.zeros_s())


def test_wallmodel_iteration_cap_is_an_error(oracle_mod):
    g, _ = _grid("les32cs")
    o = oracle_mod.Oracle(g)
    U = _smooth_field(g)
    o.set_wall_iter_cap(2)
    assert o.wallmodel(U) == -4


def _const_nu(g, nu0):
    S = g.zeros_s()
    S[1:g.n1m + 1, 1:g.n2m + 1, 1:g.n3m + 1] = nu0
    return S


def test_sgs_flux_normal_terms_modified_wavenumber(oracle_mod):
    """Constant eddy viscosity nu0, u = sin(m x) at x faces, v = cos(m' x) at cell
    centres, w = sin(m'' z) at z faces, all uniform in y: the SGS fluxes are 2 nu0 k'^2 u,
    nu0 k'^2 v and 2 nu0 k'^2 w with the (1,22,1) modified wavenumber squared
    (compact3d.f:9211).  In the two wall cells of u the d/dy(nu dv/dx) flux through the
    wall face is absent (zero wall viscosity), so u is compared inside them."""
    g, _ = _grid("les32cs")
    o = oracle_mod.Oracle(g)
    nu0 = 3.0e-3
    m1, m2, m3 = 3, 5, 2
    U = g.zeros_u()
    U[1:g.n1m + 1, :, 1:g.n3m + 1, 0] = np.sin(2 * math.pi * m1 * _xf(g) / g.alx)[:, None, None]
    U[1:g.n1m + 1, :, 1:g.n3m + 1, 1] = np.cos(2 * math.pi * m2 * _xc(g) / g.alx)[:, None, None]
    U[1:g.n1m + 1, :, 1:g.n3m + 1, 2] = np.sin(2 * math.pi * m3 * _zf(g) / g.alz)[None, None, :]
    HH = o.sgs_rhs(U, _const_nu(g, nu0))
    dx1, dx3 = g.arrays["dx1"], g.arrays["dx3"]
    slu = (slice(1, g.n1m + 1), slice(2, g.n2m), slice(1, g.n3m + 1))
    np.testing.assert_allclose(HH[slu + (0,)], 2 * nu0 * _ak(g.n1m, dx1, m1) * U[slu + (0,)], atol=1e-13)
    sl = (slice(1, g.n1m + 1), slice(1, g.n2m + 1), slice(1, g.n3m + 1))
    slv = (slice(1, g.n1m + 1), slice(2, g.n2m + 1), slice(1, g.n3m + 1))
    np.testing.assert_allclose(HH[slv + (1,)], nu0 * _ak(g.n1m, dx1, m2) * U[slv + (1,)], atol=1e-13)
    np.testing.assert_allclose(HH[sl + (2,)], 2 * nu0 * _ak(g.n3m, dx3, m3) * U[sl + (2,)], atol=1e-13)


def test_sgs_flux_wall_normal_terms_fd(oracle_mod):
    """Constant nu0 inside, zero on the wall planes; u = f(y), v = h(y), w = q(y): the
    fluxes are the second-order FD forms of d/dy(nu du/dy) (zero flux through the walls)
    and 2 d/dy(nu dv/dy)."""
    g, _ = _grid("les32cs")
    o = oracle_mod.Oracle(g)
    nu0 = 2.0e-3
    Y, DY = g.arrays["y"], g.arrays["dy"]
    H = np.concatenate([[0.0], g.arrays["h"]])   # H(1..N2) at index J
    yc = _yc(g)
    f = np.sin(1.3 * yc) + 0.2 * yc ** 2
    q = np.cos(0.7 * yc)
    yf = Y[1:g.n2m + 2]
    hv = np.sin(math.pi * yf / Y[g.n2m + 1]) * (1 + 0.3 * yf)
    U = g.zeros_u()
    U[1:g.n1m + 1, 1:g.n2m + 1, 1:g.n3m + 1, 0] = f[None, :, None]
    U[1:g.n1m + 1, 1:g.n2m + 2, 1:g.n3m + 1, 1] = hv[None, :, None]
    U[1:g.n1m + 1, 1:g.n2m + 1, 1:g.n3m + 1, 2] = q[None, :, None]
    HH = o.sgs_rhs(U, _const_nu(g, nu0))
    n2m = g.n2m
    for comp, prof in ((0, f), (2, q)):
        ext = np.concatenate([[0.0], prof, [0.0]])   # ghosts J=0, N2 are zero in U
        for J in range(1, n2m + 1):
            up = (ext[J + 1] - ext[J]) / H[J + 1] if J < n2m else 0.0
            dn = (ext[J] - ext[J - 1]) / H[J] if J > 1 else 0.0
            nup = nu0 if J < n2m else 0.0
            nud = nu0 if J > 1 else 0.0
            want = -(1.0 / DY[J]) * (nup * up - nud * dn)
            np.testing.assert_allclose(HH[1:g.n1m + 1, J, 1:g.n3m + 1, comp], want, rtol=1e-11, atol=1e-15)
    for J in range(2, n2m + 1):
        v2 = (hv[J] - hv[J - 1]) / DY[J]
        v1 = (hv[J - 1] - hv[J - 2]) / DY[J - 1]
        want = -2.0 * (1.0 / H[J]) * (nu0 * v2 - nu0 * v1)
        np.testing.assert_allclose(HH[1:g.n1m + 1, J, 1:g.n3m + 1, 1], want, rtol=1e-11, atol=1e-15)


def test_les_step_runs_and_conserves(oracle_mod):
    """A few GETUP steps of both LES models with the wall model: the field stays
    discretely divergence-free and finite, the flow rate is held, and the wall stress is
    near the log-law value of the start."""
    for name in ("les32cs", "les32dy"):
        g, dt = _grid(name)
        o = oracle_mod.Oracle(g)
        U, P, HH = ic.loglaw(g, 2000.0)
        o.project(U)
        f0 = o.chkmf(U)[0]
        S = g.zeros_s()
        pg = pg3 = 0.0
        for n in range(1, 4):
            pg, pg3 = o.getup(U, P, HH, n, dt, pg, pg3, S)
        assert np.isfinite(U).all() and np.isfinite(S).all()
        assert o.divcheck(U) < 1e-12
        assert o.chkmf(U)[0] == pytest.approx(f0, rel=1e-10)
        tw, tb, wsm = o.get_wall()
        utau = math.sqrt(wsm[0])
        assert 1500 < utau * g.re < 2600


def _loglaw_utau(U_ave, deltap, re):
    """u_tau with U_ave / u_tau = log(u_tau deltap re) / 0.41 + 5.2 (bisection to 1e-14)."""
    lo, hi = 1e-6, 1.0
    f = lambda ut: U_ave / ut - np.log(ut * deltap * re) / 0.41 - 5.2
    while hi - lo > 1e-14:
        mid = 0.5 * (lo + hi)
        if f(lo) * f(mid) <= 0:
            hi = mid
        else:
            lo = mid
    return lo


def _mesh02(g):
    y = g.arrays["y"]
    xg = np.arange(g.n1m + 2) * 0.0
    xg[1:g.n1m + 1] = np.arange(g.n1m) * g.alx / g.n1m
    xg[g.n1m + 1] = g.alx
    zg = np.zeros(g.n3m + 2)
    zg[1:g.n3m + 1] = np.arange(g.n3m) * g.alz / g.n3m
    zg[g.n3m + 1] = g.alz
    xc = 0.5 * (xg[1:] + xg[:-1])
    yc = 0.5 * (y[1:] + y[:-1])
    return xg, xc, y, yc, zg


@pytest.mark.parametrize("wmodel", [3, 5])
def test_shifted_wall_models_uniform_and_linear_fields(oracle_mod, wmodel):
    """PIOMELLI (5) and MARUSIC1 (3) on a field with uniform w, v = c y and u = a + b y
    (fields the trilinear interpolation reproduces exactly): u_tau of each wall from the
    log law on the plane-mean u of its reference plane, TAUB = u_tau^2 W / <u>, and
    TAUW = u_tau^2 + 0.1 u_tau v (PIOMELLI, v at y = H(1) and, through JPA(N2M) = N2M, at
    Y(N2M)) or
    u_tau^2 + C 0.1 u_tau (u - <u>) = u_tau^2 (MARUSIC1, u uniform on the plane)."""
    g, _ = _grid("les32cs", wmodel=wmodel)
    o = oracle_mod.Oracle(g)
    xg, xc, y, yc, zg = _mesh02(g)
    a, b, c, W = 0.4, 0.9, 0.02, 0.15
    U = g.zeros_u()
    for j in range(0, g.n2m + 2):
        yy = yc[j] if 1 <= j <= g.n2m else y[0 if j == 0 else g.n2m + 1]   # yc[J] = YC(J)
        U[:, j, :, 0] = a + b * yy
        U[:, j, :, 1] = c * y[min(j, g.n2m + 1)]
        U[:, j, :, 2] = W
    assert o.wallmodel(U) == 0
    tw, tb, wsm = o.get_wall()
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    if wmodel == 3:
        zs = [J for J in range(1, n2 + 1) if abs(y[J] - 0.06) <= abs(y[J + 1] - 0.06) and abs(y[J] - 0.06) <= abs(y[J - 1] - 0.06)][-1]
        planes, deltap = (zs, n2 - zs + 1), (yc[zs], yc[zs])
    else:
        planes, deltap = (1, n2), (g.arrays["dy"][1] / 2, g.arrays["dy"][n2] / 2)
    for wall in (0, 1):
        uave = a + b * yc[planes[wall]]
        ut = _loglaw_utau(uave, deltap[wall], g.re)
        t = tw[1:n1 + 1, 1:n3 + 1, wall]
        if wmodel == 3:
            np.testing.assert_allclose(t, ut ** 2, rtol=2e-5)
        else:
            # bottom: v between Y(1) and Y(2) at H(1); top: JPA(N2M) = N2M, so both
            # v corners are V(N2M) and the interpolant is c Y(N2M), not c YC(N2M)
            yp = g.arrays["h"][0] if wall == 0 else y[n2]
            np.testing.assert_allclose(t, ut ** 2 + 0.1 * ut * c * yp, rtol=2e-5)
        np.testing.assert_allclose(tb[1:n1 + 1, 1:n3 + 1, wall], ut ** 2 * W / uave, rtol=2e-5)
    assert wsm[0] == pytest.approx(_loglaw_utau(a + b * yc[planes[0]], deltap[0], g.re) ** 2, rel=2e-5)


def test_marusic_shift_follows_linear_u(oracle_mod):
    """MARUSIC1 samples u at XG(I) + DELTAP / tan(16 deg), wrapped into the box: with
    u = a + b y + e x on the interior x faces the interpolant is a + e XP exactly wherever
    XP falls between two interior faces, so TAUW = u_tau^2 + CC 0.1 u_tau (a + b YP + e XP
    - <u>) there, CC = 1 + 0.05 log(DY(1) / (2 DELTAP))^2 (compact3d.f:4405-4440)."""
    g, _ = _grid("les32cs", wmodel=3)
    o = oracle_mod.Oracle(g)
    xg, xc, y, yc, zg = _mesh02(g)
    a, b, e = 0.4, 0.9, 0.05
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    U = g.zeros_u()
    for j in range(0, n2 + 2):
        yy = yc[j] if 1 <= j <= n2 else y[0 if j == 0 else n2 + 1]
        U[1:n1 + 1, j, :, 0] = (a + b * yy + e * xg[1:n1 + 1])[:, None]
        U[0, j, :, 0] = U[n1, j, :, 0]
    assert o.wallmodel(U) == 0
    tw, _, _ = o.get_wall()
    zs = [J for J in range(1, n2 + 1) if abs(y[J] - 0.06) <= abs(y[J + 1] - 0.06) and abs(y[J] - 0.06) <= abs(y[J - 1] - 0.06)][-1]
    deltap = yc[zs]
    delts = deltap / math.tan(16.0 * math.pi / 180)
    cc = 1.0 + 0.05 * math.log(g.arrays["dy"][1] / 2.0 / deltap) ** 2
    checked = 0
    for wall, plane in ((0, zs), (1, n2 - zs + 1)):
        uave = a + b * yc[plane] + e * xg[1:n1 + 1].mean()
        ut = _loglaw_utau(uave, deltap, g.re)
        for i in range(1, n1 + 1):
            xp = xg[i] + delts
            if xp > g.alx:
                xp -= g.alx
            if not (xg[1] <= xp <= xg[n1]):
                continue
            want = ut ** 2 + cc * 0.1 * ut * (a + b * yc[plane] + e * xp - uave)
            # the reference's bisection stops at a bracket of 1e-7 in u_tau
            np.testing.assert_allclose(tw[i, 1:n3 + 1, wall], want, rtol=0, atol=4e-7 * ut)
            checked += 1
    assert checked >= n1


def test_dqrrt_matches_numpy_roots(oracle_mod):
    """DQRRT/CHHQR (compact3d.f:11548-11676): with a tight deflation tolerance the
    companion-matrix eigenvalues are the polynomial's roots; BETA is the largest real part
    in (0, 2), complex pairs counting by their real part, 0 when there is none.  With the
    reference's EPS = 1e-5 the deflation is early: a root moves by up to about EPS, and
    near-double roots by up to about sqrt(EPS)."""
    rng = np.random.default_rng(5)
    for _ in range(20):
        r = rng.uniform(-3.0, 3.0, 5)
        pa = np.poly(r)[1:]
        beta, ev, ok = oracle_mod.dqrrt(pa, eps=1e-14)
        assert ok == 1
        np.testing.assert_allclose(np.sort(ev.real), np.sort(r), atol=1e-7)
        inside = [x for x in r if 0.0 < x < 2.0]
        assert beta == pytest.approx(max(inside) if inside else 0.0, abs=1e-7)
        beta5, _, _ = oracle_mod.dqrrt(pa)   # near-double roots move by up to sqrt(EPS)
        assert beta5 == pytest.approx(max(inside) if inside else 0.0, abs=2e-2)
    r = np.array([0.5 + 0.3j, 0.5 - 0.3j, 1.2, -0.7, 2.5])
    beta, ev, ok = oracle_mod.dqrrt(np.real(np.poly(r))[1:], eps=1e-14)
    np.testing.assert_allclose(np.sort_complex(ev), np.sort_complex(r), atol=1e-7)
    assert beta == pytest.approx(1.2, abs=1e-9)
    r = np.array([0.6 + 0.3j, 0.6 - 0.3j, 0.2, -0.7, 2.5])
    beta, _, _ = oracle_mod.dqrrt(np.real(np.poly(r))[1:], eps=1e-14)
    assert beta == pytest.approx(0.6, abs=1e-9)


@pytest.mark.parametrize("four", [False, True])
def test_filters_on_fourier_modes(oracle_mod, four):
    """FILTER multiplies a mode cos(a x + b z) by (4 + 2 cos a)(4 + 2 cos b) / 36 and
    FILTER4 (compact3d.f:5481-5545) by (2 + 8 cos a + 2 cos 2a)(2 + 8 cos b + 2 cos 2b)
    / 144, a and b the mode's phase steps per cell."""
    g, _ = _grid("les32dy")
    o = oracle_mod.Oracle(g)
    n1, n3 = g.n1m, g.n3m
    i, k = np.meshgrid(np.arange(n1), np.arange(n3))
    F = np.stack([np.cos(2 * np.pi * (mx * i / n1 + mz * k / n3)) for mx, mz in ((1, 0), (3, 2), (5, 7))])
    out = o.filter(F, four)
    for q, (mx, mz) in enumerate(((1, 0), (3, 2), (5, 7))):
        a, b = 2 * np.pi * mx / n1, 2 * np.pi * mz / n3
        if four:
            gain = (2 + 8 * np.cos(a) + 2 * np.cos(2 * a)) * (2 + 8 * np.cos(b) + 2 * np.cos(2 * b)) / 144
        else:
            gain = (4 + 2 * np.cos(a)) * (4 + 2 * np.cos(b)) / 36
        np.testing.assert_allclose(out[q], gain * F[q], atol=1e-14)


def test_sgssd_invariances(oracle_mod):
    """SGSSD (compact3d.f:1502-1948): the Germano sums are quartic in the velocity, so the
    quintic and BETA are unchanged when U is scaled, SGSVIS scales with U (where it is
    not clipped), and a uniform velocity added to the field changes nothing (the filters
    have unit weight sums)."""
    g, _ = _grid("les32dy", files=3, wmodel=0, cks=2.0)
    o = oracle_mod.Oracle(g)
    U, P, HH = ic.loglaw(g, 2000.0)
    o.project(U)
    S0, sm0 = o.sgs(U)
    b0 = o.get_beta()
    assert np.all((b0 > 0) & (b0 < 2))
    S1, sm1 = o.sgs(2.5 * U)
    np.testing.assert_allclose(o.get_beta(), b0, rtol=1e-9)
    np.testing.assert_allclose(sm1, sm0, rtol=1e-8)
    sl = (slice(1, g.n1m + 1), slice(1, g.n2m + 1), slice(1, g.n3m + 1))
    unclipped = 2.5 * S0[sl] > -1.0 / g.re
    np.testing.assert_allclose(S1[sl][unclipped], 2.5 * S0[sl][unclipped], rtol=1e-8, atol=1e-20)
    U2 = U.copy(order="F")
    U2[..., 0] += 0.3
    U2[..., 2] -= 0.2
    S2, sm2 = o.sgs(U2)
    np.testing.assert_allclose(o.get_beta(), b0, rtol=1e-8)
    np.testing.assert_allclose(S2[sl], S0[sl], rtol=1e-8, atol=1e-14)


def test_sgssd_step_runs_and_conserves(oracle_mod):
    g, dt = _grid("les32dy", files=3)
    o = oracle_mod.Oracle(g)
    U, P, HH = ic.loglaw(g, 2000.0)
    o.project(U)
    f0 = o.chkmf(U)[0]
    S = g.zeros_s()
    pg = pg3 = 0.0
    for n in range(1, 4):
        pg, pg3 = o.getup(U, P, HH, n, dt, pg, pg3, S)
    assert np.isfinite(U).all() and np.isfinite(S).all()
    assert o.divcheck(U) < 1e-12
    assert o.chkmf(U)[0] == pytest.approx(f0, rel=1e-10)
    assert np.all((o.get_beta() >= 0) & (o.get_beta() < 2))


# --- WALLMODEL_IWMLES_SMOOTH (WMODEL 2): a numpy restatement of one model update ---
_IW = {n: q for q, n in enumerate(
    "UTX UTY TAUWX TAUWY FTX FTY FTMX FTMY FP I0 I1 I2 I3 I4 M0 M1 M2 M3 M4 DIFFX DIFFY LHSX LHSY FUS TR DZ "
    "AX AY CX CY UNSX UNSY DELI DELV DTX DTY DBX DBY CONVX CONVY PRSX PRSY".split())}


def _iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty, re):
    vonk, reinv = 0.4, 1.0 / re
    us = (utx ** 4 + uty ** 4) ** 0.25
    delv, deli = reinv / us, min(11.0 * reinv / us, Dz)
    Vel = math.sqrt(Ux ** 2 + Uy ** 2)
    lg = math.log(deli / Dz)
    Ax = (Ux / us + Ux / Vel / vonk * lg - deli / delv * utx / us) / (1 - deli / Dz)
    Ay = (Uy / us + Uy / Vel / vonk * lg - deli / delv * uty / us) / (1 - deli / Dz)
    Cx, Cy = Ux / us - Ax, Uy / us - Ay
    Lu = 0.5 * utx * deli ** 2 / delv + us * Dz * (0.5 * Ax * (1 - deli ** 2 / Dz ** 2) + Cx * (1 - deli / Dz)
                                                   - Ux / Vel / vonk * (1 - deli / Dz + deli / Dz * lg))
    Lv = 0.5 * uty * deli ** 2 / delv + us * Dz * (0.5 * Ay * (1 - deli ** 2 / Dz ** 2) + Cy * (1 - deli / Dz)
                                                   - Uy / Vel / vonk * (1 - deli / Dz + deli / Dz * lg))
    return Lu + lhsx, Lv + lhsy


def _iwm_loglaw(U_ave, dz, re):
    u1, u2, lam = 1.0, 1e-6, 1.0
    while abs(u2 - u1) > 1e-6:
        u1 = u2
        f1 = U_ave / u1 - math.log(u1 * dz * re) / 0.4 - 5.0
        f2 = -U_ave / u1 ** 2 - 1.0 / 0.4 / u1
        u2 = u1 - lam * f1 / f2
        if abs(U_ave / u2 - math.log(u2 * dz * re) / 0.4 - 5.0) > abs(f1):
            lam *= 0.5
    return u1


def _iwm_update(g, st, U, P, wm_dt, presg, presg3):
    """One update of iwm_calc_lhs_smooth and iwm_calc_wallstress_smooth
    (compact3d.f:3718-4279); st is (slots, N3M, N1M), modified in place."""
    n1, n3, re, vonk = g.n1m, g.n3m, g.re, 0.4
    reinv = 1.0 / re
    S = {n: st[q] for n, q in _IW.items()}
    u_inst = U[1:n1 + 1, 3, 1:n3 + 1, 0].T
    v_inst = U[1:n1 + 1, 3, 1:n3 + 1, 2].T
    p_inst = P[:n1, 0, :n3].T
    p_inst = p_inst - p_inst.sum() / n1 / n3
    S["FTMX"][:] = S["FTX"]
    S["FTMY"][:] = S["FTY"]
    tR = S["TR"].copy()
    S["FTX"][:] = S["FTX"] * (1 - tR) + u_inst * tR
    S["FTY"][:] = S["FTY"] * (1 - tR) + v_inst * tR
    S["FP"][:] = S["FP"] * (1 - tR) + p_inst * tR
    dx1, dx3 = g.arrays["dx1"], g.arrays["dx3"]
    dxf = lambda a: (np.roll(a, -1, 1) - np.roll(a, 1, 1)) * dx1 / 2.0
    dzf = lambda a: (np.roll(a, -1, 0) - np.roll(a, 1, 0)) * dx3 / 2.0
    ux, vy = dxf(S["I0"]), dzf(S["I2"])
    S["CONVX"][:] = dxf(S["I1"]) + dzf(S["I4"]) - S["FTMX"] * (ux + vy)
    S["CONVY"][:] = dxf(S["I4"]) + dzf(S["I3"]) - S["FTMY"] * (ux + vy)
    S["PRSX"][:] = dxf(S["FP"]) * S["DZ"] + presg * S["DZ"]
    S["PRSY"][:] = dzf(S["FP"]) * S["DZ"] + presg3 * S["DZ"]
    S["LHSX"][:] = -S["I0"] + wm_dt * (S["CONVX"] + S["PRSX"] - S["DIFFX"])
    S["LHSY"][:] = -S["I2"] + wm_dt * (S["CONVY"] + S["PRSY"] - S["DIFFY"])
    deltap = g.arrays["dy"][1] + g.arrays["dy"][2] + g.arrays["dy"][3] / 2.0
    eqx = eqy = 0.0
    for i in range(n1):
        for k in range(n3):
            lhsx, lhsy, Ux, Uy, Dz = S["LHSX"][k, i], S["LHSY"][k, i], S["FTX"][k, i], S["FTY"][k, i], S["DZ"][k, i]
            utx, uty = S["UTX"][k, i], S["UTY"][k, i]
            fx, fy = _iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty, re)
            it, eq = 0, 0
            while max(abs(fx), abs(fy)) > 1e-6:
                e = 1e-9
                fxp, fyp = _iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx + e, uty, re)
                a11, a21 = (fxp - fx) / e, (fyp - fy) / e
                fxp, fyp = _iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty + e, re)
                a12, a22 = (fxp - fx) / e, (fyp - fy) / e
                det = a11 * a22 - a12 * a21
                utx, uty = utx - (a22 * fx - a12 * fy) / det, uty - (-a21 * fx + a11 * fy) / det
                fx, fy = _iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty, re)
                it += 1
                if it > 1500:
                    eq = 1
                    break
            if utx - 1.0 == utx or uty - 1.0 == uty:
                eq = 1
            if eq:
                U_ave = math.sqrt(Ux ** 2 + Uy ** 2)
                t1 = _iwm_loglaw(U_ave, deltap, re) ** 2
                eqx, eqy = t1 * Ux / U_ave, t1 * Uy / U_ave
                utx, uty = math.sqrt(abs(eqx)), math.sqrt(abs(eqy))
            px, py = utx, uty
            ut = (px ** 4 + py ** 4) ** 0.25
            delv, deli = reinv / ut, min(11 * reinv / ut, Dz)
            Vel = math.sqrt(Ux ** 2 + Uy ** 2)
            lg = math.log(deli / Dz)
            Ax = Ay = Cx = Cy = 0.0
            if not eq:
                Ax = (Ux / ut + Ux / Vel / vonk * lg - deli / delv * px / ut) / (1 - deli / Dz)
                Ay = (Uy / ut + Uy / Vel / vonk * lg - deli / delv * py / ut) / (1 - deli / Dz)
                Cx, Cy = Ux / ut - Ax, Uy / ut - Ay
            if abs(Ax) > 1.0 or abs(Ay) > 1.0:
                eq = 1
                utx, uty = math.sqrt(abs(eqx)), math.sqrt(abs(eqy))
                Ax = Ay = Cx = Cy = 0.0
            S["UTX"][k, i], S["UTY"][k, i] = utx, uty
            r1, r2, r3 = deli / Dz, deli ** 2 / Dz ** 2, deli ** 3 / Dz ** 3
            lu = lambda pu, A, C, Uc: 0.5 * pu * deli ** 2 / delv + ut * Dz * (
                0.5 * A * (1 - r2) + C * (1 - r1) - Uc / Vel / vonk * (1 - r1 + r1 * lg))
            luu = lambda pu, A, C, Uc: pu ** 2 * deli ** 3 / delv ** 2 / 3 + ut ** 2 * Dz * (
                -A * Uc / Vel / vonk * r2 * lg + A * (C - Uc / Vel / 2 / vonk) * (1 - r2) + A ** 2 / 3 * (1 - r3)
                + (C - Uc / Vel / vonk) ** 2 - r1 * (C - Uc / Vel / vonk + Uc / Vel / vonk * lg) ** 2
                + Uc ** 2 / Vel ** 2 / vonk ** 2 * (1 - r1))
            S["M0"][k, i], S["M1"][k, i], S["M2"][k, i], S["M3"][k, i], S["M4"][k, i] = (
                S["I0"][k, i], S["I1"][k, i], S["I2"][k, i], S["I3"][k, i], S["I4"][k, i])
            S["I0"][k, i] = lu(px, Ax, Cx, Ux)
            S["I2"][k, i] = lu(py, Ay, Cy, Uy)
            S["I1"][k, i] = luu(px, Ax, Cx, Ux)
            S["I3"][k, i] = luu(py, Ay, Cy, Uy)
            S["I4"][k, i] = px * py * deli ** 3 / delv ** 2 / 3 + ut ** 2 * Dz * (
                -(Ax * Uy / Vel + Ay * Ux / Vel) / vonk * (0.25 - 0.25 * r2 + 0.5 * deli ** 2 / Dz * lg)
                - (Cx * Uy / Vel + Cy * Ux / Vel) / vonk * (1 - r1 + r1 * lg)
                - Ux * Uy / Vel ** 2 / vonk ** 2 * (r1 - 2 + r1 * (lg - 1) ** 2)
                + Ax * Ay / 3 * (1 - r3) + 0.5 * (Ax * Cy + Ay * Cx) * (1 - r2) + Cx * Cy * (1 - r1))
            if deli < Dz:
                dTx, dTy = ut / Dz * (Ax + Ux / Vel / vonk), ut / Dz * (Ay + Uy / Vel / vonk)
            else:
                dTx, dTy = px / delv, py / delv
            dBx, dBy = px / delv, py / delv
            dV = abs(Ux / Vel * dTx + Uy / Vel * dTy)
            if deli < Dz:
                S["DIFFX"][k, i] = (reinv + (vonk * Dz) ** 2 * dV) * dTx - reinv * dBx
                S["DIFFY"][k, i] = (reinv + (vonk * Dz) ** 2 * dV) * dTy - reinv * dBy
            else:
                S["DIFFX"][k, i] = S["DIFFY"][k, i] = 0.0
            if eq:
                S["TAUWX"][k, i], S["TAUWY"][k, i] = eqx, eqy
            elif deli < Dz:
                S["TAUWX"][k, i], S["TAUWY"][k, i] = px ** 2, py ** 2
            else:
                S["TAUWX"][k, i], S["TAUWY"][k, i] = reinv * Ux / Dz, reinv * Uy / Dz
            S["FUS"][k, i] = S["FUS"][k, i] * (1 - S["TR"][k, i]) + ut * S["TR"][k, i]
            S["TR"][k, i] = min(wm_dt / (Dz / S["FUS"][k, i] / vonk), 1.0)


@pytest.mark.parametrize("n2m", [16, 64])
def test_iwmles_update_matches_numpy_restatement(oracle_mod, n2m):
    """WALLMODEL_IWMLES_SMOOTH: the state after the first two model updates (steps 5 and
    10) against a numpy restatement applied to the state, field and pressure the oracle
    held before each update; steps 1-4 impose the initial u_tau^2 (from the log law on the
    plane-mean u of plane 3), the spanwise stress in TAUB, and WSM(1) is the mean stress."""
    g, dt = _grid("les32cs", wmodel=2, n2m=n2m)
    o = oracle_mod.Oracle(g)
    o.set_cflmax(0.5)
    U, P, HH = ic.loglaw(g, 2000.0)
    o.project(U)
    S = g.zeros_s()
    pg = pg3 = 0.0
    dzp = g.arrays["dy"][1] + g.arrays["dy"][2] + g.arrays["dy"][3] / 2.0
    uinit = U[1:g.n1m + 1, 3, 1:g.n3m + 1, 0].mean()
    us0 = _iwm_loglaw(uinit, dzp, g.re)
    for n in range(1, 11):
        if n % 5 == 0:
            st = o.get_iwm().copy()
            U0, P0 = U.copy(), P.copy()
            pgs, pg3s = pg, pg3
        pg, pg3 = o.getup(U, P, HH, n, dt, pg, pg3, S)
        tw, tb, wsm = o.get_wall()
        if n < 5:
            np.testing.assert_allclose(tw[1:g.n1m + 1, 1:g.n3m + 1, 0], us0 ** 2, rtol=1e-12)
            assert np.abs(tb[1:g.n1m + 1, 1:g.n3m + 1, 0]).max() == 0.0
            assert wsm[0] == pytest.approx(us0 ** 2, rel=1e-12)
        if n % 5 == 0:
            # the reference's stale fallback leaves u_tau = 0 at points, after which its
            # formulas divide by zero: the restatement follows them through inf and NaN
            with np.errstate(divide="ignore", invalid="ignore"):
                _iwm_update(g, st, U0, P0, 5 * dt, pgs, pg3s)
            got = o.get_iwm()
            for name in ("UTX", "UTY", "TAUWX", "TAUWY", "FTX", "FTY", "FP", "I0", "I1", "I2", "I3", "I4", "DIFFX",
                         "DIFFY", "LHSX", "LHSY", "FUS", "TR"):
                q = _IW[name]
                np.testing.assert_allclose(got[q], st[q], rtol=1e-9, atol=1e-13 * max(1.0, np.abs(st[q]).max()),
                                           err_msg=name)
            np.testing.assert_allclose(tw[1:g.n1m + 1, 1:g.n3m + 1, 0], got[_IW["TAUWX"]].T, rtol=0, atol=0)
            np.testing.assert_allclose(tb[1:g.n1m + 1, 1:g.n3m + 1, 0], got[_IW["TAUWY"]].T, rtol=0, atol=0)
            assert wsm[0] == pytest.approx(np.mean(np.sqrt(got[_IW["TAUWX"]] ** 2 + got[_IW["TAUWY"]] ** 2)),
                                           rel=1e-12, abs=1e-300)
    assert np.isfinite(U).all()


def test_rough_wall_model_log_law(oracle_mod):
    """WALLMODEL_ROUGH (WMODEL 1 with Y0 = Y(0) != 0, compact3d.f:2496-2558): TAUW1 =
    (0.41 |U| / log(DELTAP / Y0))^2 along the velocity of plane 3 per bottom-wall point,
    WSM(1) its plane mean, DELTAP = DY(1) + DY(2) + DY(3)/2."""
    g, _ = _grid("les32cs", y0=2e-3)
    o = oracle_mod.Oracle(g)
    U, P, HH = ic.loglaw(g, 2000.0)
    assert o.wallmodel(U) == 0
    tw, tb, wsm = o.get_wall()
    dy = g.arrays["dy"]
    dp = dy[1] + dy[2] + dy[3] / 2.0
    u, w = U[1:g.n1m + 1, 3, 1:g.n3m + 1, 0], U[1:g.n1m + 1, 3, 1:g.n3m + 1, 2]
    mag = np.sqrt(u ** 2 + w ** 2)
    t1 = (0.41 / math.log(dp / 2e-3) * mag) ** 2
    np.testing.assert_allclose(tw[1:g.n1m + 1, 1:g.n3m + 1, 0], t1 * u / mag, rtol=1e-13)
    np.testing.assert_allclose(tb[1:g.n1m + 1, 1:g.n3m + 1, 0], t1 * w / mag, rtol=1e-13)
    assert wsm[0] == pytest.approx(t1.mean(), rel=1e-13)


def test_iwmles_rough_initial_stress(oracle_mod):
    """WALLMODEL_IWMLES_ROUGH (WMODEL 2 with Y0 != 0, compact3d.f:2562-3381): until the first
    update the imposed stress is u_tau^2 with u_tau = 0.4 <u(3)> / log(Dzp / Y0)
    (iwm_init_rough), the spanwise stress is 0, and the updates keep the field finite."""
    g, dt = _grid("les32cs", wmodel=2, y0=1e-3)
    o = oracle_mod.Oracle(g)
    o.set_cflmax(0.5)
    U, P, HH = ic.loglaw(g, 2000.0)
    o.project(U)
    dzp = g.arrays["dy"][1] + g.arrays["dy"][2] + g.arrays["dy"][3] / 2.0
    us0 = U[1:g.n1m + 1, 3, 1:g.n3m + 1, 0].mean() * 0.4 / math.log(dzp / 1e-3)
    S = g.zeros_s()
    pg = pg3 = 0.0
    for n in range(1, 12):
        pg, pg3 = o.getup(U, P, HH, n, dt, pg, pg3, S)
        tw, tb, wsm = o.get_wall()
        if n < 5:
            np.testing.assert_allclose(tw[1:g.n1m + 1, 1:g.n3m + 1, 0], us0 ** 2, rtol=1e-12)
            assert np.abs(tb[1:g.n1m + 1, 1:g.n3m + 1, 0]).max() == 0.0
    assert np.isfinite(U).all() and np.isfinite(tw).all()

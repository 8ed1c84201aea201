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

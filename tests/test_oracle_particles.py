"""Known answers for the oracle's restatement of the particle step (CALC_UX_4RK,
FORCE_PAR, BC_PAR's deterministic part) and SOURCE_PAR (compact3d.f:2029-2075,
11882-12470): in a uniform flow the interpolated fluid velocity is exact, so one step is
a classical RK4 step of the drag-gravity ODE, which numpy repeats."""
import math

import numpy as np
import pytest

from compact3d_gb300.grid import make_grid

DIAM, DENS, HHH = 0.0002, 2220.0, 0.05


def _uniform(g, u0, w0):
    U = g.zeros_u()
    U[..., 0] = u0
    U[..., 2] = w0
    return U


def _force(re, up, vp, wp, uf, vf, wf):
    D = DIAM / HHH
    tau = DENS * D ** 2 / 18.0 * re
    rep = math.sqrt((uf - up) ** 2 + (vf - vp) ** 2 + (wf - wp) ** 2) * D * re
    with np.errstate(divide="ignore"):
        fcor = 1.0 + 0.15 * rep ** 0.687 + 0.0175 / (1.0 + 42500.0 * np.float64(rep) ** -1.16)
    g = -9.8 / (0.000015 * re / HHH) ** 2
    return fcor * (uf - up) / tau, fcor * (vf - vp) / tau + g, fcor * (wf - wp) / tau


def _rk4(re, p, dt, uf, wf):
    k = []
    s = np.array(p, dtype=float)
    for c in (0.5, 0.5, 1.0, None):
        q = _force(re, s[3], s[4], s[5], uf, 0.0, wf)
        k.append(np.array([s[3], s[4], s[5], *q]))
        if c is None:
            break
        s = np.array(p) + c * dt * k[-1]
    return np.array(p) + dt * (k[0] + 2 * k[1] + 2 * k[2] + k[3]) / 6.0


def test_rk4_step_in_uniform_flow(oracle_mod):
    g, dt = make_grid("les32cs", wmodel=3)
    o = oracle_mod.Oracle(g)
    U = _uniform(g, 0.7, 0.1)
    par = np.array([[1.3, 0.4, 2.0, 0.2, 0.05, 0.0], [3.0, 1.2, 0.5, 0.9, -0.02, 0.3], [7.1, 0.9, 9.0, 0.0, 0.0, 0.0]])
    out, imp = o.particles_advance(U, par, dt, DIAM, DENS, HHH)
    for q in range(len(par)):
        np.testing.assert_allclose(out[q], _rk4(g.re, par[q], dt, 0.7, 0.1), rtol=1e-12, atol=1e-14)
    assert not imp.any()


def test_periodic_shift_and_top_reflection(oracle_mod):
    g, dt = make_grid("les32cs", wmodel=3)
    o = oracle_mod.Oracle(g)
    D = DIAM / HHH
    U = _uniform(g, 0.0, 0.0)
    # leaves through x = ALX: BC_PAR shifts it by ALX - D; one at the top moving up reflects
    par = np.array([[g.alx - 0.5 * D - 1e-6, 1.0, 1.0, 1.0, 0.0, 0.0]])
    out, _ = o.particles_advance(U, par, dt, DIAM, DENS, HHH)
    x_free = _rk4(g.re, par[0], dt, 0.0, 0.0)[0]
    assert out[0, 0] == pytest.approx(D + x_free - g.alx, abs=1e-12)
    top = np.array([[2.0, 2.0 - 0.5 * D - 1e-9, 1.0, 0.0, 0.5, 0.0]])
    out, _ = o.particles_advance(U, top, dt, DIAM, DENS, HHH)
    # the first stage already starts outside: the explicit Euler step, then the reflection
    ye = top[0, 1] + dt * 0.5
    assert out[0, 4] < 0 and out[0, 1] == pytest.approx(2.0 * 2.0 - D - ye, abs=1e-12)


def test_bottom_impact_flagged_and_source_terms(oracle_mod):
    g, dt = make_grid("les32cs", wmodel=3)
    o = oracle_mod.Oracle(g)
    D = DIAM / HHH
    U = _uniform(g, 0.5, 0.0)
    par = np.array([[1.0, 0.5 * D + 1e-7, 1.0, 0.0, -1.0, 0.0]])
    _, imp = o.particles_advance(U, par, dt, DIAM, DENS, HHH)
    assert imp[0] == 1
    # SOURCE_PAR: one particle's drag at the u, v, w points of its cell
    # (gravity and G cancel for a particle moving with the fluid vertically: VISCOS =
    # 1.5e-5, so the v term is the drag alone)
    p = np.array([[1.0, 0.7, 2.0, 0.2, -0.1, 0.0]])
    r1, r2, r3 = o.particles_source(U, p, DIAM, DENS, HHH)
    mass = DENS * 3.141592653 * D ** 3 / 6.0
    qu, qv, qw = _force(g.re, 0.2, -0.1, 0.0, 0.5, 0.0, 0.0)
    gg = 9.8 / (g.re * 1.5 / 100000 / HHH) ** 2
    dx1, dx3 = g.arrays["dx1"], g.arrays["dx3"]
    nz = np.argwhere(r1 != 0)
    assert len(nz) == 1 and len(np.argwhere(r2 != 0)) == 1 and np.abs(r3).max() == 0.0
    i, j, k = nz[0]
    assert r1[i, j, k] == pytest.approx(-mass * 1000.0 * qu * dx1 * dx3 / g.arrays["h"][j - 1], rel=1e-12)
    i2, j2, k2 = np.argwhere(r2 != 0)[0]
    assert r2[i2, j2, k2] == pytest.approx(-mass * 1000.0 * (qv + gg) * dx1 * dx3 / g.arrays["h"][j2 - 1], rel=1e-12)

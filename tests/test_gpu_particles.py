"""The particle step and SOURCE_PAR's terms on the device against the oracle: a random
cloud in a perturbed log-law field, FP64 and mixed channels (the particle arithmetic is
FP64 in both; the mixed state is double-float), positions and velocities within 1e-12
relative after five steps (FP64; pow in FORCE_PAR may differ in the last bit), source
terms within 1e-12 of their largest value."""
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


@pytest.mark.parametrize("prec,tol", [(C3D_FP64, 1e-12), (C3D_MIXED, 1e-9)])
def test_particles_match_oracle(libc3d, oracle_mod, prec, tol):
    g, dt = make_grid("les32cs", wmodel=3)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.loglaw(g, 2000.0)
    orc.project(U)
    ch = libc3d.Channel(g, prec)
    ch.upload(U, P, HH)
    rng = np.random.default_rng(11)
    n = 3000
    D = 0.0002 / 0.05
    par = np.column_stack([rng.uniform(0, g.alx, n), rng.uniform(0.5 * D, 2.0 - 0.5 * D, n), rng.uniform(0, g.alz, n),
                           rng.normal(0.5, 0.2, n), rng.normal(0, 0.05, n), rng.normal(0, 0.05, n)])
    par[:50, 1] = rng.uniform(0.5 * D, 3 * D, 50)       # near the bottom wall: impacts and Euler steps
    par[:50, 4] = -np.abs(par[:50, 4]) - 0.5
    par[50:100, 1] = 2.0 - rng.uniform(0.5 * D, 3 * D, 50)   # near the top wall: reflections
    par[50:100, 4] = np.abs(par[50:100, 4]) + 0.5
    a, b = par.copy(), par.copy()
    for _ in range(5):
        a, ia = ch.particles_advance(a, dt)
        b, ib = orc.particles_advance(U, b, dt)
        np.testing.assert_array_equal(ia, ib)
    assert ib.sum() > 0
    for c in range(6):
        # particles left below the bottom wall (handed to SPLASH in the reference) carry NaN
        np.testing.assert_allclose(a[:, c], b[:, c], rtol=tol, atol=tol * np.nanmax(np.abs(b[:, c])))
    sa, sb = ch.particles_source(par), orc.particles_source(U, par)
    for x, y in zip(sa, sb):
        assert np.abs(x - y).max() <= tol * np.abs(y).max()
        assert np.abs(y).max() > 0

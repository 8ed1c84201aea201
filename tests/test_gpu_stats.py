"""ENERGY's plane statistics on the device (c3d_plane_stats) against the oracle's
restatement: FP64 form 1e-12 relative per column (FP64 sums in another order), mixed
form 1e-6 (its state is double-float; the statistics are still taken in FP64)."""
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


def _col_err(a, b):
    return np.max(np.linalg.norm(a - b, axis=0) / np.maximum(np.linalg.norm(b, axis=0), 1e-300))


@pytest.mark.parametrize("prec,tol", [(C3D_FP64, 1e-12), (C3D_MIXED, 1e-6)])
def test_plane_stats_match_oracle(libc3d, oracle_mod, prec, tol):
    g, dt = make_grid("small32", n1m=64, n2m=32, n3m=64)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g, amp=0.3)
    orc.project(U)
    pg = pg3 = 0.0
    for m in (1, 2):
        pg, pg3 = orc.getup(U, P, HH, m, dt, pg, pg3)
    ch = libc3d.Channel(g, prec)
    ch.upload(U, P, HH)
    s = ch.plane_stats()
    ref = orc.plane_stats(U, P)
    cols = [q for q in range(29) if np.linalg.norm(ref[:, q]) > 1e-10]
    assert _col_err(s[:, cols], ref[:, cols]) < tol
    small = [q for q in range(29) if q not in cols]
    assert np.abs(s[:, small]).max() < 1e-8
    assert s.shape == (g.n2m, 29)


@pytest.mark.parametrize("prec,tol", [(C3D_FP64, 1e-12), (C3D_MIXED, 1e-6)])
@pytest.mark.parametrize("shape", [dict(n1m=64, n2m=32, n3m=64), dict(n1m=96, n2m=16, n3m=48)])
def test_plane_spectra_match_oracle(libc3d, oracle_mod, prec, tol, shape):
    """ENERGY's spectra and correlations (c3d_plane_spectra) against the oracle: relative
    L2 per (plane, component) line of each table, FP64 1e-12 (FP64 FFTs of other orders
    than the oracle's), mixed 1e-6; with the instantaneous means and with a given VMO.
    The correlations divide by VRMS - VM^2, which cancels where the mean dominates (u:
    mean near 1, variance near 1e-4), so their FP64 bound is 1e-10."""
    g, dt = make_grid("small32", **shape)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g, amp=0.3)
    orc.project(U)
    pg = pg3 = 0.0
    for m in (1, 2):
        pg, pg3 = orc.getup(U, P, HH, m, dt, pg, pg3)
    ch = libc3d.Channel(g, prec)
    ch.upload(U, P, HH)
    rng = np.random.default_rng(3)
    vmo = orc.plane_stats(U, P)[:, 0:3] + 1e-3 * rng.standard_normal((g.n2m, 3))
    for v in (None, vmo):
        a, b = ch.plane_spectra(v), orc.plane_spectra(U, v)
        for key in ("xspec", "zspec", "rxx", "rzz", "rxy"):
            x, y = a[key], b[key]
            assert x.shape == y.shape
            err = np.linalg.norm(x - y, axis=0) / np.maximum(np.linalg.norm(y, axis=0), 1e-300)
            bound = max(tol, 1e-10) if key.startswith("r") else tol
            assert err.max() < bound, (key, err.max())


@pytest.mark.parametrize("prec", [C3D_FP64, C3D_MIXED])
def test_plane_quadrants_match_oracle(libc3d, oracle_mod, prec):
    """Quadrant analysis (c3d_plane_quadrants) against the oracle, with VMP = the plane
    means and with the reference's zero VMP: FP64 sums 1e-12, point fractions exact; the
    mixed form's double-float state may move a point that sits within rounding of an axis,
    so its fractions get one point per plane of slack and its sums 1e-6."""
    g, dt = make_grid("small32", n1m=64, n2m=32, n3m=64)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g, amp=0.3)
    orc.project(U)
    ch = libc3d.Channel(g, prec)
    ch.upload(U, P, HH)
    vmp = orc.plane_stats(U, P)[:, 0:2]
    for v in (vmp, None):
        a, b = ch.plane_quadrants(v), orc.plane_quadrants(U, v)
        if prec == C3D_FP64:
            np.testing.assert_allclose(a[:, :4], b[:, :4], rtol=1e-12, atol=1e-18)
            np.testing.assert_array_equal(a[:, 4:], b[:, 4:])
        else:
            assert np.abs(a[:, :4] - b[:, :4]).max() <= 1e-6 * np.abs(b[:, :4]).max()
            assert np.abs(a[:, 4:] - b[:, 4:]).max() <= 1.0 / (g.n1m * g.n3m) + 1e-15


@pytest.mark.parametrize("prec", [C3D_FP64, C3D_MIXED])
def test_wall_spectrum_and_corr3d_match_oracle(libc3d, oracle_mod, prec):
    """SPECTAUW (c3d_wall_spectrum) and RXYZ (c3d_corr3d) against the oracle: the wall
    spectrum is FP64 on the FP64 wall stress in both forms (1e-12 relative to its peak);
    RXYZ 1e-10 (FP64, VRMS - VM^2 cancels) and 1e-6 (mixed) relative L2 per component."""
    g, dt = make_grid("small32", n1m=64, n2m=32, n3m=48)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g, amp=0.3)
    orc.project(U)
    ch = libc3d.Channel(g, prec)
    ch.upload(U, P, HH)
    rng = np.random.default_rng(4)
    tw = np.zeros(g.shape_tau(), order="F")
    tw[1:g.n1m + 1, 1:g.n3m + 1, :] = 2.5e-3 + 1e-4 * rng.standard_normal((g.n1m, g.n3m, 2))
    tb = np.asfortranarray(0.1 * tw)
    orc.set_wall(tw, tb, 1)
    ch.upload_wall(tw, tb)
    a, b = ch.wall_spectrum(0.05), orc.wall_spectrum(0.05)
    assert np.abs(a - b).max() < 1e-12 * np.abs(b).max()
    r, q = ch.corr3d(), orc.corr3d(U)
    tol = 1e-10 if prec == C3D_FP64 else 1e-6
    for L in range(3):
        assert np.linalg.norm(r[..., L] - q[..., L]) < tol * np.linalg.norm(q[..., L]), L

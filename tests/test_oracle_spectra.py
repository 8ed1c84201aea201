"""Known answers for the FP64 oracle's restatement of ENERGY's 1-D spectra and two-point
correlations (compact3d.f:10243-10515) on single Fourier modes."""
import math

import numpy as np
import pytest

from compact3d_gb300.grid import make_grid


def _mode_field(g, mx, mz, A=0.3, phase=0.4):
    """u(I,J,K) = U0(J) + A cos(2 pi (mx (I-1)/N1M + mz (K-1)/N3M) + phase) at the x faces."""
    U = g.zeros_u()
    i = np.arange(g.n1m)[:, None]
    k = np.arange(g.n3m)[None, :]
    wave = A * np.cos(2 * np.pi * (mx * i / g.n1m + mz * k / g.n3m) + phase)
    for j in range(1, g.n2m + 1):
        U[1:g.n1m + 1, j, 1:g.n3m + 1, 0] = 0.5 + 0.01 * j + wave
    U[0, :, :, 0] = U[g.n1m, :, :, 0]
    U[:, :, 0, 0] = U[:, :, g.n3m, 0]
    return U


def test_x_mode_spectrum_and_correlation(oracle_mod):
    g, _ = make_grid("tiny16")
    o = oracle_mod.Oracle(g)
    m, A = 3, 0.3
    U = _mode_field(g, m, 0, A)
    r = o.plane_spectra(U)
    n = g.n1m
    # the cell-centre average of a face mode: amplitude A cos(pi m / N), phase + pi m / N
    Ac = A * math.cos(math.pi * m / n)
    fs = math.pi * g.arrays["dx1"]
    want = np.zeros(n)
    want[m] = want[n - m] = Ac ** 2 * n / 4 / fs
    for j in range(g.n2m):
        np.testing.assert_allclose(r["xspec"][:, j, 0], want, atol=1e-13)
    assert np.abs(r["xspec"][:, :, 1:]).max() < 1e-25
    # z spectrum of a field constant in z: only k = 0, |sum_K (u_c - VM)|^2 per line
    zk0 = r["zspec"][0, :, 0]
    assert np.abs(r["zspec"][1:, :, 0]).max() < 1e-24 and zk0.max() > 0
    theta = 2 * np.pi * m * (np.arange(n) + 0.5) / n + 0.4
    n1h = n // 2 + 1
    np.testing.assert_allclose(r["rxx"][:, 3, 0], 2 * np.cos(theta[n1h - 1]) * np.cos(theta), atol=1e-12)
    np.testing.assert_allclose(r["rxy"][:, 3, 0], 2 * np.cos(theta[n1h - 1]) * np.cos(theta), atol=1e-12)


def test_z_mode_spectrum_and_correlation(oracle_mod):
    g, _ = make_grid("tiny16")
    o = oracle_mod.Oracle(g)
    m, A = 2, 0.25
    U = _mode_field(g, 0, m, A)
    vmo = np.zeros((g.n2m, 3))
    vmo[:, 0] = [0.5 + 0.01 * (j + 1) for j in range(g.n2m)]
    r = o.plane_spectra(U, vmo)
    n = g.n3m
    fs = math.pi * g.arrays["dx3"]
    want = np.zeros(n)
    want[m] = want[n - m] = A ** 2 * n / 4 / fs
    for j in range(g.n2m):
        np.testing.assert_allclose(r["zspec"][:, j, 0], want, atol=1e-13)
    theta = 2 * np.pi * m * np.arange(n) / n + 0.4
    n3h = n // 2 + 1
    np.testing.assert_allclose(r["rzz"][:, 5, 0], 2 * np.cos(theta[n3h - 1]) * np.cos(theta), atol=1e-12)
    # each x line is constant: only k = 0, N1M <wave^2> / (PI DX1) = N1M A^2 / 2 / (PI DX1)
    assert np.abs(r["xspec"][1:, :, 0]).max() < 1e-24
    np.testing.assert_allclose(r["xspec"][0, :, 0], g.n1m * A ** 2 / 2 / (math.pi * g.arrays["dx1"]), rtol=1e-12)


def test_quadrants_of_a_correlated_mode(oracle_mod):
    """Quadrant analysis (compact3d.f:10560-10604): u' = a cos(theta), v' = b cos(theta)
    about VMP put every point in quadrant 1 or 3 with u'v' = a b cos^2: Q(1) = Q(3) =
    -a b / 4, QP(1) = QP(3) = 1/2; with VMP = 0 (the reference's unset local) and u > 0
    everywhere the points fall in quadrants 1 and 4 by the sign of v."""
    g, _ = make_grid("tiny16")
    o = oracle_mod.Oracle(g)
    a, b, c = 0.3, 0.2, 0.5
    U = g.zeros_u()
    theta = 2 * np.pi * 3 * (np.arange(g.n1m) + 0.5) / g.n1m + 0.1
    xf = 2 * np.pi * 3 * np.arange(g.n1m) / g.n1m + 0.1
    # u at the x faces whose centre average is c + a cos(theta): a' = a / cos(pi m / N)
    ap = a / math.cos(math.pi * 3 / g.n1m)
    U[1:g.n1m + 1, :, 1:g.n3m + 1, 0] = (c + ap * np.cos(xf))[:, None, None]
    U[1:g.n1m + 1, :, 1:g.n3m + 1, 1] = (b * np.cos(theta))[:, None, None]
    vmp = np.zeros((g.n2m, 2))
    vmp[:, 0] = c
    q = o.plane_quadrants(U, vmp)
    np.testing.assert_allclose(q[:, 0], -a * b / 4, rtol=1e-12)
    np.testing.assert_allclose(q[:, 2], -a * b / 4, rtol=1e-12)
    np.testing.assert_allclose(q[:, [1, 3]], 0.0, atol=1e-15)
    np.testing.assert_allclose(q[:, [4, 6]], 0.5, rtol=1e-12)
    q0 = o.plane_quadrants(U)
    np.testing.assert_allclose(q0[:, 4] + q0[:, 7], 1.0, rtol=1e-12)
    np.testing.assert_allclose(q0[:, 0] + q0[:, 3], -np.mean((c + a * np.cos(theta)) * b * np.cos(theta)), rtol=1e-12)


def test_time_average_follows_taver():
    """TimeAverage is TAVER's running mean: the first sample copied, then
    (XO (NAVG-1) + X) / NAVG, which equals the arithmetic mean up to rounding."""
    from compact3d_gb300.lib import TimeAverage
    rng = np.random.default_rng(2)
    xs = [rng.standard_normal((5, 3)) for _ in range(7)]
    ta = TimeAverage()
    ref = None
    for n, x in enumerate(xs, 1):
        m = ta.add(stats=x)["stats"]
        ref = x.copy() if n == 1 else (ref * (n - 1.0) + x) / n
        np.testing.assert_array_equal(m, ref)
    np.testing.assert_allclose(m, np.mean(xs, axis=0), rtol=1e-13)
    with pytest.raises(ValueError):
        ta.add(other=xs[0])


def test_wall_spectrum_and_corr3d_known_answers(oracle_mod):
    """SPECTAUW of TAUW = UTAU^2 + A cos(2 pi (m i / N1M + n k / N3M)) has its two peaks
    A^2 N1M N3M / 4 / (PI DX1) / (PI DX3) at (m, n) and (-m, -n); RXYZ of an x mode is
    2 cos(theta(N1H)) cos(theta(I)) on every plane and z index."""
    g, _ = make_grid("tiny16")
    o = oracle_mod.Oracle(g)
    utau, A, m, n = 0.05, 1e-3, 2, 3
    i = np.arange(g.n1m)[:, None]
    k = np.arange(g.n3m)[None, :]
    tw = np.zeros(g.shape_tau(), order="F")
    tw[1:g.n1m + 1, 1:g.n3m + 1, 0] = utau ** 2 + A * np.cos(2 * np.pi * (m * i / g.n1m + n * k / g.n3m))
    o.set_wall(tw, np.zeros(g.shape_tau(), order="F"), 1)
    s = o.wall_spectrum(utau)
    want = np.zeros((g.n1m, g.n3m))
    peak = A ** 2 * g.n1m * g.n3m / 4 / (math.pi * g.arrays["dx1"]) / (math.pi * g.arrays["dx3"])
    want[m, n] = want[g.n1m - m, g.n3m - n] = peak
    np.testing.assert_allclose(s, want, atol=1e-12 * peak)
    U = _mode_field(g, 3, 0, 0.3)
    r = o.corr3d(U)
    theta = 2 * np.pi * 3 * (np.arange(g.n1m) + 0.5) / g.n1m + 0.4
    want3 = 2 * np.cos(theta[g.n1m // 2]) * np.cos(theta)
    np.testing.assert_allclose(r[:, 4, 7, 0], want3, atol=1e-12)
    np.testing.assert_allclose(r[:, 0, 2, 0], want3, atol=1e-12)

"""Known-answer tests that pin the FP64 CPU oracle.

The reference ships no tests or golden vectors and cannot be built here, so the oracle is
checked against closed-form answers and independent implementations:
  1. FFT against numpy.fft (FFTW conventions: forward exponent -1, unnormalised);
  2. the cyclic solvers CTDMA11 / CTDMA1J against dense numpy solves;
  3. the compact operators (1,6,1), (1,10,1), (1,22,1) against their analytic modified
     wavenumbers, and AK1/AK3 against 288 dx^-2 (1-cos t)/(11+cos t)^2 (compact3d.f:9211);
  4. the Poisson solve as the exact inverse of div(grad): a projected field has
     max|div| at rounding level (DIVCHECK), and GETDP(div grad p) recovers p;
  5. a laminar Poiseuille start stays laminar, keeps its flow rate, and settles to the
     laminar pressure gradient -2/RE.
"""
import math

import numpy as np
import pytest

from compact3d_gb300 import ic
from compact3d_gb300.grid import make_grid


@pytest.mark.parametrize("n", [8, 16, 24, 48, 64, 96, 128, 192, 256, 384])
def test_fft_matches_numpy(oracle_mod, n):
    rng = np.random.default_rng(n)
    z = rng.normal(size=n) + 1j * rng.normal(size=n)
    f = oracle_mod.fft(z, -1)
    assert np.abs(f - np.fft.fft(z)).max() <= 1e-14 * np.abs(np.fft.fft(z)).max() * math.log2(n)
    b = oracle_mod.fft(z, +1)
    assert np.abs(b - n * np.fft.ifft(z)).max() <= 1e-14 * np.abs(b).max() * math.log2(n)


def test_dft2d_fortran_order(oracle_mod):
    rng = np.random.default_rng(7)
    a = np.asfortranarray(rng.normal(size=(48, 32)) + 1j * rng.normal(size=(48, 32)))
    f = oracle_mod.dft2d(a, -1)
    assert np.allclose(f, np.fft.fft2(a), rtol=0, atol=1e-12 * np.abs(f).max())


def _circulant(n, a, b, c):
    M = np.zeros((n, n))
    for i in range(n):
        M[i, i] = b
        M[i, (i - 1) % n] = a
        M[i, (i + 1) % n] = c
    return M


@pytest.mark.parametrize("n", [16, 48, 64, 96, 384])
@pytest.mark.parametrize("abc", [(1, 6, 1), (1, 10, 1), (1, 22, 1), (0.9987, 10.0026, 0.9987)])
def test_cyclic_solvers_dense(oracle_mod, n, abc):
    rng = np.random.default_rng(n)
    d = rng.normal(size=n)
    x = np.linalg.solve(_circulant(n, *abc), d)
    assert np.abs(oracle_mod.ctdma11(d, *abc) - x).max() < 1e-14 * np.abs(x).max() * 10
    assert np.abs(oracle_mod.ctdma_recip(d, *abc) - x).max() < 1e-14 * np.abs(x).max() * 10


def test_tdmap_dense(oracle_mod):
    rng = np.random.default_rng(3)
    n = 40
    a, c = rng.uniform(0.5, 1, n), rng.uniform(0.5, 1, n)
    b = -(a + c) - rng.uniform(0.1, 1, n)
    r = rng.normal(size=n)
    M = np.diag(b) + np.diag(a[1:], -1) + np.diag(c[:-1], 1)
    assert np.allclose(oracle_mod.tdmap(a, b, c, r), np.linalg.solve(M, r), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("n", [32, 96])
def test_compact_modified_wavenumbers(oracle_mod, n):
    dx1 = n / (2 * math.pi)
    for m in (1, 3, n // 6, n // 3):
        t = 2 * math.pi * m / n
        i = np.arange(n)
        f = np.cos(t * i)
        # first derivative at faces: (1,22,1) X = 24 DX1 (f_i - f_{i-1})
        d = 24 * dx1 * (f - np.roll(f, 1))
        x = oracle_mod.ctdma11(d, 1, 22, 1)
        kmod = 48 * dx1 * math.sin(t / 2) / (22 + 2 * math.cos(t))
        assert np.allclose(x, -kmod * np.sin(t * (i - 0.5)), atol=1e-12 * kmod)
        # second derivative: (1,10,1) X = 12 DX1^2 (f_{i-1} - 2 f_i + f_{i+1})
        d = 12 * dx1 ** 2 * (np.roll(f, 1) - 2 * f + np.roll(f, -1))
        x = oracle_mod.ctdma11(d, 1, 10, 1)
        k2 = 12 * dx1 ** 2 * (2 - 2 * math.cos(t)) / (10 + 2 * math.cos(t))
        assert np.allclose(x, -k2 * f, atol=1e-12 * k2)
        # interpolation to faces: (1,6,1) X = 4 (f_{i-1} + f_i)
        d = 4 * (np.roll(f, 1) + f)
        x = oracle_mod.ctdma11(d, 1, 6, 1)
        g = 8 * math.cos(t / 2) / (6 + 2 * math.cos(t))
        assert np.allclose(x, g * np.cos(t * (i - 0.5)), atol=1e-13)


def test_poisson_wavenumbers(oracle_mod):
    g, _ = make_grid("small32")
    orc = oracle_mod.Oracle(g)
    ak1, ak3, pm, pc, pp = orc.poisson_metrics()
    dx1, dx3 = g.arrays["dx1"], g.arrays["dx3"]
    for I in range(1, g.n1m + 1):
        m = I - 1 if I <= g.n1m // 2 + 1 else I - 1 - g.n1m
        t = 2 * math.pi * m / g.n1m
        assert ak1[I - 1] == pytest.approx(288 * dx1 ** 2 * (1 - math.cos(t)) / (11 + math.cos(t)) ** 2,
                                           rel=1e-13, abs=1e-12)
    for K in range(1, g.n3m // 2 + 2):
        t = 2 * math.pi * (K - 1) / g.n3m
        assert ak3[K - 1] == pytest.approx(288 * dx3 ** 2 * (1 - math.cos(t)) / (11 + math.cos(t)) ** 2,
                                           rel=1e-13, abs=1e-12)
    # interior rows of the y operator sum to zero (Neumann-type walls)
    assert np.allclose(pm + pc + pp, 0, atol=1e-9 * np.abs(pc).max())


@pytest.mark.parametrize("name", ["tiny16", "small32"])
def test_projection_is_divergence_free(oracle_mod, name):
    g, _ = make_grid(name)
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.bcond(U)
    assert orc.divcheck(U) > 1e-6
    orc.project(U)
    assert orc.divcheck(U) < 1e-12


def test_getdp_inverts_div_grad(oracle_mod):
    """GETDP(L p) = p, with L = div(grad) built from the same discrete operators."""
    g, _ = make_grid("tiny16")
    orc = oracle_mod.Oracle(g)
    rng = np.random.default_rng(11)
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    p = rng.normal(size=(n1, n2, n3))
    p -= p[:, 0, :].mean()                  # (kx,kz)=(0,0) mode pinned at J=1
    dx1, dx3 = g.arrays["dx1"], g.arrays["dx3"]
    H = g.arrays["h"]
    UH = g.zeros_u()
    for j in range(n2):
        for k in range(n3):
            UH[1:n1 + 1, j + 1, k + 1, 0] = oracle_mod.ctdma11(24 * dx1 * (p[:, j, k] - np.roll(p[:, j, k], 1)), 1, 22, 1)
        for i in range(n1):
            UH[i + 1, j + 1, 1:n3 + 1, 2] = oracle_mod.ctdma11(24 * dx3 * (p[i, j, :] - np.roll(p[i, j, :], 1)), 1, 22, 1)
    for j in range(1, n2):   # faces J=2..N2M
        UH[1:n1 + 1, j + 1, 1:n3 + 1, 1] = (p[:, j, :] - p[:, j - 1, :]) / H[j]
    rdp = orc.rhsdp(UH, 1.0)
    dp = orc.getdp(rdp)
    assert np.abs(dp[:n1, :n2, :n3] - p).max() < 1e-10 * np.abs(p).max()


def test_laminar_start_stays_laminar(oracle_mod):
    g, dt = make_grid("tiny16")
    orc = oracle_mod.Oracle(g)
    U = g.zeros_u()
    Y = g.arrays["y"]
    yc = 0.5 * (Y[1:g.n2m + 1] + Y[2:g.n2m + 2])
    U[1:g.n1m + 1, 1:g.n2m + 1, 1:g.n3m + 1, 0] = (yc * (2 - yc))[None, :, None]
    P, HH = g.zeros_p(), g.zeros_u()
    f0 = orc.chkmf(U)[0]
    pg = pg3 = 0.0
    for n in range(1, 301):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
    u = U[1:g.n1m + 1, 1:g.n2m + 1, 1:g.n3m + 1]
    assert np.abs(u[..., 1]).max() < 1e-12 and np.abs(u[..., 2]).max() < 1e-12
    assert np.abs(u[..., 0] - u[:1, :, :1, 0]).max() < 1e-12      # x-z uniform
    assert orc.chkmf(U)[0] == pytest.approx(f0, rel=1e-12)
    assert pg == pytest.approx(-2.0 / g.re, rel=0.05)
    assert abs(pg3) < 1e-14


def test_flow_rate_conserved_turbulent_start(oracle_mod):
    g, dt = make_grid("small32")
    orc = oracle_mod.Oracle(g)
    U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    f0 = orc.chkmf(U)[0]
    pg = pg3 = 0.0
    for n in range(1, 11):
        pg, pg3 = orc.getup(U, P, HH, n, dt, pg, pg3)
        assert orc.divcheck(U) < 1e-11
    assert orc.chkmf(U)[0] == pytest.approx(f0, rel=1e-11)


def test_plane_stats_laminar_profile(oracle_mod):
    """ENERGY's plane statistics of a laminar profile u = U(y), v = w = 0: the moments of a
    constant plane (uu = u^2, central moments 0), wz = -dU/dy at the cell centres with
    ENERGY's interpolants, and pressure statistics of a plane-constant P."""
    from compact3d_gb300.grid import make_grid
    g, _ = make_grid("small32")
    o = oracle_mod.Oracle(g)
    U = g.zeros_u()
    y = g.arrays["y"]
    yc = 0.5 * (y[1:g.n2m + 1] + y[2:g.n2m + 2])
    for j in range(0, g.n2m + 2):
        yy = yc[j - 1] if 1 <= j <= g.n2m else (y[1] if j == 0 else y[g.n2m + 1])
        U[:, j, :, 0] = yy * (2.0 - yy)
    P = g.zeros_p()
    P[:, :g.n2m, :] = np.arange(g.n2m)[None, :, None] * 0.1
    s = o.plane_stats(U, P)
    u = s[:, 0]
    np.testing.assert_allclose(s[:, 7], u * u, rtol=1e-13)
    assert np.abs(s[:, [1, 2, 8, 9, 10, 11, 12, 18, 19, 20, 21, 22, 23, 24, 25]]).max() < 1e-20
    np.testing.assert_allclose(s[:, 6], -s[:, 26], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(s[:, 3], np.arange(g.n2m) * 0.1, atol=1e-15)
    np.testing.assert_allclose(s[:, 13], (np.arange(g.n2m) * 0.1) ** 2, atol=1e-15)

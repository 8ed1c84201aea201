"""Seeded synthetic initial conditions for the channel workloads.

The reference's INIUP (compact3d.f:503-723) draws unseeded uniform noise, so its
initial fields cannot be reproduced.  This module builds seeded fields instead:

* ``perturbed_laminar``: the laminar profile of INIUP (``REALU``, compact3d.f:612) plus
  ``amp`` times the curl of a band-limited random vector potential that vanishes with
  zero slope at both walls, so the perturbation is divergence-free in the continuous
  sense and zero at the walls.  It is then made discretely divergence-free by one
  pressure projection (``c3d_project`` in the library, ``orc_project`` in the oracle).
* ``loglaw``: the wall-modelled LES start: a log-law mean profile (Reichardt's composite
  law of the wall, u+ = ln(1 + 0.41 y+)/0.41 + 7.8 (1 - exp(-y+/11) - y+/11 exp(-y+/3)),
  with y+ from the nearest wall) plus ``amp`` times its centreline value in the same
  divergence-free perturbation as ``perturbed_laminar``.
* ``band_limited``: seeded N(0,1) fields band-limited to |k| <= N/3 in x and z with a
  smooth random wall-normal profile (the operator workload).

All fields use the reference's Fortran layouts (U(0:N1,0:N2,0:N3,3), P(N1,N2,N3)).
"""
from __future__ import annotations

import numpy as np

from .grid import Grid

SEED0 = 20261203


def _spectral_field(rng, n1m, n3m, kx_max, kz_max):
    """Random real trig polynomial on (x,z); returns its rfft2 spectrum S[kz, kx]."""
    S = np.zeros((n3m, n1m // 2 + 1), dtype=np.complex128)
    for mz in range(-kz_max, kz_max + 1):
        for mx in range(0, kx_max + 1):
            if mx == 0 and mz <= 0:
                continue
            S[mz % n3m, mx] = rng.normal() + 1j * rng.normal()
    return S


def _eval(S, n1m, n3m, sx, sz, dx_order=0, dz_order=0):
    """Values of the field (or its x/z derivative, in units of the domain being
    2*pi*[1/Lx..]) at x=(i+sx)*dx, z=(k+sz)*dz; returns array [k, i]."""
    kx = np.arange(n1m // 2 + 1)
    kz = np.fft.fftfreq(n3m, 1.0 / n3m)
    ph = np.exp(2j * np.pi * (kx[None, :] * sx / n1m + kz[:, None] * sz / n3m))
    T = S * ph
    if dx_order:
        T = T * (1j * kx[None, :]) ** dx_order
    if dz_order:
        T = T * (1j * kz[:, None]) ** dz_order
    return np.fft.irfft2(T, s=(n3m, n1m)) * (n1m * n3m)


def perturbed_laminar(g: Grid, amp: float = 0.1, seed: int = SEED0, kmax: int = 4, mean=None):
    """U, P, HH (Fortran order) of the perturbed laminar start (before projection).
    ``mean`` (a function of the cell-centre y array) replaces the laminar profile; the
    perturbation is then scaled to ``amp`` times the profile's maximum."""
    rng = np.random.default_rng(seed)
    n1m, n2m, n3m = g.n1m, g.n2m, g.n3m
    a = g.arrays
    Y = a["y"]
    aly = a["aly"]
    yc = 0.5 * (Y[1:n2m + 1] + Y[2:n2m + 2])          # cell centres J=1..N2M
    yf = Y[1:n2m + 2]                                   # faces J=1..N2
    kx2 = 2 * np.pi / g.alx
    kz2 = 2 * np.pi / g.alz
    kxm = min(kmax, n1m // 3)
    kzm = min(kmax, n3m // 3)
    F = [_spectral_field(rng, n1m, n3m, kxm, kzm) for _ in range(3)]

    def env(y):
        s = y * (2.0 - y)
        return s * s

    def denv(y):
        s = y * (2.0 - y)
        return 2.0 * s * (2.0 - 2.0 * y)

    # u at (x=(i-1)dx, yc, z=(k-1/2)dz): d psi3/dy - d psi2/dz
    F3u = _eval(F[2], n1m, n3m, 0.0, 0.5)
    dzF2u = _eval(F[1], n1m, n3m, 0.0, 0.5, dz_order=1) * kz2
    pu = denv(yc)[:, None, None] * F3u[None] - env(yc)[:, None, None] * dzF2u[None]
    # v at (x=(i-1/2)dx, y face, zc): d psi1/dz - d psi3/dx
    dzF1v = _eval(F[0], n1m, n3m, 0.5, 0.5, dz_order=1) * kz2
    dxF3v = _eval(F[2], n1m, n3m, 0.5, 0.5, dx_order=1) * kx2
    pv = env(yf)[:, None, None] * (dzF1v - dxF3v)[None]
    # w at (xc, yc, z=(k-1)dz): d psi2/dx - d psi1/dy
    dxF2w = _eval(F[1], n1m, n3m, 0.5, 0.0, dx_order=1) * kx2
    F1w = _eval(F[0], n1m, n3m, 0.5, 0.0)
    pw = env(yc)[:, None, None] * dxF2w[None] - denv(yc)[:, None, None] * F1w[None]
    U = g.zeros_u()
    if mean is None:
        realu = yc * (aly - yc) * (aly - 1.0) + yc * (2 * aly - yc) * (2.0 - aly)
        ref = 1.0
    else:
        realu = mean(yc)
        ref = float(np.abs(realu).max())
    scale = amp * ref / max(np.abs(pu).max(), np.abs(pv).max(), np.abs(pw).max(), 1e-300)
    # arrays pu[j,k,i] -> U[i,j,k]
    U[1:n1m + 1, 1:n2m + 1, 1:n3m + 1, 0] = (realu[:, None, None] + scale * pu).transpose(2, 0, 1)
    U[1:n1m + 1, 1:n2m + 2, 1:n3m + 1, 1] = (scale * pv).transpose(2, 0, 1)
    U[1:n1m + 1, 1, 1:n3m + 1, 1] = 0.0
    U[1:n1m + 1, n2m + 1, 1:n3m + 1, 1] = 0.0
    U[1:n1m + 1, 1:n2m + 1, 1:n3m + 1, 2] = (scale * pw).transpose(2, 0, 1)
    P = g.zeros_p()
    HH = g.zeros_u()
    return U, P, HH


def loglaw(g: Grid, retau: float, amp: float = 0.05, seed: int = SEED0, kmax: int = 4):
    """U, P, HH of the LES start: Reichardt's law of the wall at friction Reynolds number
    ``retau`` (u_tau = retau / RE in the reference's units) plus a divergence-free
    perturbation of ``amp`` times the centreline velocity."""
    utau = retau / g.re
    aly = g.arrays["aly"]

    def prof(y):
        yw = np.minimum(y, aly - y) if aly == 2.0 else y
        yp = yw * retau
        up = np.log1p(0.41 * yp) / 0.41 + 7.8 * (1.0 - np.exp(-yp / 11.0) - yp / 11.0 * np.exp(-yp / 3.0))
        return utau * up

    return perturbed_laminar(g, amp=amp, seed=seed, kmax=kmax, mean=prof)


def band_limited(g: Grid, seed: int = SEED0, frac: float = 1.0 / 3.0):
    """Seeded N(0,1) fields band-limited to |k| <= frac*N in x and z, times a smooth
    random y-profile (sum of 4 Chebyshev modes).  Returns U (3 comps) and P."""
    rng = np.random.default_rng(seed)
    n1m, n2m, n3m = g.n1m, g.n2m, g.n3m
    Y = g.arrays["y"]
    yc = 0.5 * (Y[1:n2m + 1] + Y[2:n2m + 2])
    t = yc / g.arrays["aly"] * 2 - 1
    out = []
    for _ in range(4):
        f = rng.normal(size=(n2m, n3m, n1m))
        S = np.fft.rfft2(f, axes=(1, 2))
        kx = np.arange(n1m // 2 + 1)
        kz = np.abs(np.fft.fftfreq(n3m, 1.0 / n3m))
        mask = (kx[None, :] <= frac * n1m / 2) & (kz[:, None] <= frac * n3m / 2)
        S *= mask[None]
        f = np.fft.irfft2(S, s=(n3m, n1m), axes=(1, 2))
        c = rng.normal(size=4)
        prof = sum(c[m] * np.cos(m * np.arccos(np.clip(t, -1, 1))) for m in range(4))
        f = f * prof[:, None, None]
        f /= max(np.abs(f).max(), 1e-300)
        out.append(f)
    U = g.zeros_u()
    U[1:n1m + 1, 1:n2m + 1, 1:n3m + 1, 0] = out[0].transpose(2, 0, 1)
    U[1:n1m + 1, 2:n2m + 1, 1:n3m + 1, 1] = out[1][1:].transpose(2, 0, 1)
    U[1:n1m + 1, 1:n2m + 1, 1:n3m + 1, 2] = out[2].transpose(2, 0, 1)
    P = g.zeros_p()
    P[:n1m, :n2m, :n3m] = out[3].transpose(2, 0, 1)
    return U, P

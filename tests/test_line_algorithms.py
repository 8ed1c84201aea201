"""CPU checks of the algorithms the CUDA kernels use for the compact line solves.

The kernels factor the constant-coefficient cyclic operator tridiag(a, b, a) as
(-a/r)(1 - rS)(1 - rS^-1) and evaluate two first-order recurrences.  These numpy models
follow the device code step by step (lane chunks with affine warp scans along x, the
general form and the constant-multiplier form of row segments of 8, 16 or 32 lanes;
segments with a warm-up of M points along z) and are compared with the oracle's
bordered-LU solver (CTDMA11, compact3d.f:8952-8998).
"""
import math

import numpy as np
import pytest


def coeffs(a, b, fp32=False):
    beta = b / a
    r = -2.0 / (beta + math.sqrt(beta * beta - 4.0))
    s = -r / a
    m = math.ceil(math.log(3e-8 if fp32 else 1e-17) / math.log(abs(r)))
    return r, s, m


def xsolve_model(d, a, b):
    """Warp of 32 lanes, lane l owns C = ceil(n/32) consecutive points."""
    n = len(d)
    C = -(-n // 32)
    P = n // C
    r, s, _ = coeffs(a, b)
    x = [list(d[l * C:(l + 1) * C]) if l < P else [0.0] * C for l in range(32)]
    # forward local
    e, m = [0.0] * 32, [1.0] * 32
    for l in range(P):
        y, mm = 0.0, 1.0
        for t in range(C):
            y = x[l][t] + r * y
            mm *= r
        e[l], m[l] = y, mm
    # inclusive Hillis-Steele scan of affine maps
    off = 1
    while off < 32:
        e2, m2 = e[:], m[:]
        for l in range(32):
            if l >= off:
                e2[l] = e[l] + m[l] * e[l - off]
                m2[l] = m[l] * m[l - off]
        e, m = e2, m2
        off *= 2
    y0 = e[31] / (1 - m[31])
    for l in range(P):
        y = y0 if l == 0 else e[l - 1] + m[l - 1] * y0
        for t in range(C):
            y = x[l][t] + r * y
            x[l][t] = y
    # backward
    e, m = [0.0] * 32, [1.0] * 32
    for l in range(P):
        z, mm = 0.0, 1.0
        for t in reversed(range(C)):
            z = x[l][t] + r * z
            mm *= r
        e[l], m[l] = z, mm
    off = 1
    while off < 32:
        e2, m2 = e[:], m[:]
        for l in range(32):
            if l + off < 32:
                e2[l] = e[l] + m[l] * e[l + off]
                m2[l] = m[l] * m[l + off]
        e, m = e2, m2
        off *= 2
    z0 = e[0] / (1 - m[0])
    out = np.zeros(n)
    for l in range(P):
        z = z0 if l == 31 else e[l + 1] + m[l + 1] * z0
        for t in reversed(range(C)):
            z = x[l][t] + r * z
            out[l * C + t] = s * z
    return out


def xsolve_full_model(d, a, b, W):
    """A row held by a segment of W lanes with every lane holding a chunk of C = n/W points
    (the device's xsolve_full): the scans combine with the constant multipliers
    r^(C 2^b), lane l closes with r^(C l) (forward) and r^(C (W-1-l)) (backward), formed
    from the bits of l, and the cyclic closure divides by 1 - r^(C W) only when that
    power is not below half an ulp."""
    n = len(d)
    assert n % W == 0
    C = n // W
    lw = W.bit_length() - 1
    r, s, _ = coeffs(a, b)
    pw = [1.0]
    for _ in range(C):
        pw[0] *= r
    for q in range(lw):
        pw.append(pw[q] * pw[q])
    ml = [math.prod(pw[q] for q in range(lw) if (l >> q) & 1) for l in range(W)]
    mr = [math.prod(pw[q] for q in range(lw) if ((W - 1 - l) >> q) & 1) for l in range(W)]
    exact1 = abs(pw[lw]) < 2.0 ** -54
    x = [list(d[l * C:(l + 1) * C]) for l in range(W)]
    e = []
    for l in range(W):
        y = 0.0
        for t in range(C):
            y = x[l][t] + r * y
        e.append(y)
    for q in range(lw):
        off = 1 << q
        e = [e[l] + pw[q] * e[l - off] if l >= off else e[l] for l in range(W)]
    y0 = e[W - 1] if exact1 else e[W - 1] / (1.0 - pw[lw])
    for l in range(W):
        y = y0 if l == 0 else e[l - 1] + ml[l] * y0
        for t in range(C):
            y = x[l][t] + r * y
            x[l][t] = y
    e = []
    for l in range(W):
        z = 0.0
        for t in reversed(range(C)):
            z = x[l][t] + r * z
        e.append(z)
    for q in range(lw):
        off = 1 << q
        e = [e[l] + pw[q] * e[l + off] if l + off < W else e[l] for l in range(W)]
    z0 = e[0] if exact1 else e[0] / (1.0 - pw[lw])
    out = np.zeros(n)
    for l in range(W):
        z = z0 if l == W - 1 else e[l + 1] + mr[l] * z0
        for t in reversed(range(C)):
            z = x[l][t] + r * z
            out[l * C + t] = s * z
    return out


def zseg_model(d, a, b, L=16):
    n = len(d)
    r, s, M = coeffs(a, b)
    out = np.zeros(n)
    for k0 in range(0, n, L):
        y = 0.0
        for q in range(k0 - M, k0):
            y = d[q % n] + r * y
        ys = []
        for t in range(L):
            y = d[(k0 + t) % n] + r * y
            ys.append(y)
        acc, pw = 0.0, 1.0
        for q in range(M):
            y = d[(k0 + L + q) % n] + r * y
            acc += pw * y
            pw *= r
        z = acc
        for t in reversed(range(L)):
            z = ys[t] + r * z
            out[k0 + t] = s * z
    return out


@pytest.mark.parametrize("n", [16, 32, 48, 64, 96, 128, 192, 256, 384])
@pytest.mark.parametrize("ab", [(1.0, 6.0), (1.0, 10.0), (1.0, 22.0), (0.9985, 10.003)])
def test_warp_scan_solver(oracle_mod, n, ab):
    d = np.random.default_rng(n).normal(size=n)
    ref = oracle_mod.ctdma11(d, ab[0], ab[1], ab[0])
    assert np.abs(xsolve_model(d, *ab) - ref).max() < 4e-15 * np.abs(ref).max()


@pytest.mark.parametrize("n,W", [(16, 8), (48, 8), (64, 8), (96, 8), (128, 16), (64, 32), (384, 32)])
@pytest.mark.parametrize("ab", [(1.0, 6.0), (1.0, 10.0), (1.0, 22.0), (0.9985, 10.003)])
def test_constant_multiplier_segment_solver(oracle_mod, n, ab, W):
    """The row-segment line solve with constant scan multipliers, for the row lengths and
    segment widths the kernels use (and a 16-point row, where r^(C W) is not negligible
    and the closure divides)."""
    d = np.random.default_rng(n + W).normal(size=n)
    ref = oracle_mod.ctdma11(d, ab[0], ab[1], ab[0])
    assert np.abs(xsolve_full_model(d, *ab, W) - ref).max() < 4e-15 * np.abs(ref).max()


@pytest.mark.parametrize("n", [16, 48, 64, 384])
@pytest.mark.parametrize("ab", [(1.0, 6.0), (1.0, 22.0), (0.9985, 10.003)])
def test_segment_warmup_solver(oracle_mod, n, ab):
    d = np.random.default_rng(n + 1).normal(size=n)
    ref = oracle_mod.ctdma11(d, ab[0], ab[1], ab[0])
    assert np.abs(zseg_model(d, *ab) - ref).max() < 4e-15 * np.abs(ref).max()


def test_warmup_lengths():
    # |r|^M below the FP64 / FP32 rounding units for the three Pade operators
    for b in (6.0, 10.0, 22.0):
        for fp32, tol in ((False, 1e-17), (True, 3e-8)):
            r, _, m = coeffs(1.0, b, fp32)
            assert abs(r) ** m <= tol

"""GPU parity of the isolated operators (c3d_op_*) against the oracle's restatement of
the reference routines (CTDMA11/CTDMA33 with the RHS1/RHS2 right-hand sides, the y
stencils, GETDP).

Tolerances (relative L2 over the planes each operator writes):
  * FP64 form: 1e-13 for the line solves and stencils, 1e-11 for the Poisson solve
    (a different FFT and solve order on a near-singular mean mode);
  * mixed form (FP32 operand and result; double-float Poisson recurrences): 2e-6 for the
    line solves and stencils, 2e-5 for the Poisson solve.
"""
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


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def operand(g, seed=11):
    """A band-limited field F(0:M1,0:M2,0:M3) with non-zero wall planes."""
    U, P = ic.band_limited(g, seed=seed)
    F = np.asfortranarray(U[..., 0])
    rng = np.random.default_rng(seed)
    F[1:g.n1m + 1, 0, 1:g.n3m + 1] = rng.normal(size=(g.n1m, g.n3m))
    F[1:g.n1m + 1, g.n2m + 1, 1:g.n3m + 1] = rng.normal(size=(g.n1m, g.n3m))
    return F


def written(g, op, X):
    j0 = 2 if op == 7 else 1
    return X[1:g.n1m + 1, j0:g.n2m + 1, 1:g.n3m + 1]


@pytest.mark.parametrize("name", ["small32", "channel64"])
def test_operators_fp64_match_oracle(libc3d, oracle_mod, name):
    g, _ = make_grid(name)
    orc = oracle_mod.Oracle(g)
    ch = libc3d.Channel(g, C3D_FP64)
    F = operand(g)
    for key, op in libc3d.OPS.items():
        Xg = ch.operator(op, F)
        Xo = orc.operator(op, F)
        tol = 1e-11 if key == "POISSON" else 1e-13
        e = rel(written(g, op, Xg), written(g, op, Xo))
        assert e < tol, (key, e)


def test_operators_mixed_error(libc3d, oracle_mod):
    g, _ = make_grid("channel64")
    orc = oracle_mod.Oracle(g)
    ch = libc3d.Channel(g, C3D_MIXED)
    F = operand(g, seed=5)
    for key, op in libc3d.OPS.items():
        e = rel(written(g, op, ch.operator(op, F)), written(g, op, orc.operator(op, F)))
        assert e < (2e-5 if key == "POISSON" else 2e-6), (key, e)


def test_operator_repeat_is_idempotent(libc3d):
    """c3d_op_apply(count) recomputes the result from the same operand each time."""
    g, _ = make_grid("small32")
    ch = libc3d.Channel(g, C3D_FP64)
    F = operand(g)
    ch.op_set(F)
    ch.op_apply(libc3d.OPS["DZ1"], 1)
    a = ch.op_get()
    ch.op_apply(libc3d.OPS["DZ1"], 5)
    b = ch.op_get()
    assert np.array_equal(a, b)

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

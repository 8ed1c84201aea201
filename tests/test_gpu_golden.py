"""GPU parity against golden fixtures of the reference's own GETUP.

tests/golden/*.npz were made by tests/golden/make_golden.py from compact3d.f itself,
translated to C (oracle/f77c.py) because no Fortran compiler exists here: the seeded,
projected start, and the state after three GETUP steps (compact3d.f:879-960), with the
diagnostics of the last state.  The CUDA library starts from the same inputs through the
C-ABI and must land on the reference's state:

  * FP64 form: relative L2 1e-10 for u, v, w and HH, 1e-10 for P, SGSVIS and the wall
    stresses (LES); PRESG to 1e-8 relative (a difference of two channel-wide sums
    divided by DT, so its summation order matters at that level); DIVCHECK's
    max|div u| within 1e-13 absolute, CFL and CHKMF to 1e-12;
  * mixed form: 2e-5 for u, v, w after the three steps.
"""
import os

import numpy as np
import pytest

from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, make_grid

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [("tiny16_dns.npz", "tiny16", {}, False), ("les16_les.npz", "les32cs", dict(n1m=16, n3m=16), True)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def interior(g, U, P, HH):
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    return dict(u=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0], v=U[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1],
                w=U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2], p=P[:n1, :n2, :n3], hh=HH[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, :])


@pytest.fixture(scope="module")
def libc3d():
    from compact3d_gb300 import build, lib
    build.build()
    lib.load()
    return lib


def run(libc3d, fname, name, over, les, precision):
    d = np.load(os.path.join(GOLDEN, fname))
    g, dt = make_grid(name, **over)
    assert float(d["dt"]) == dt
    ch = libc3d.Channel(g, precision)
    ch.upload(*(np.asfortranarray(d[k]) for k in ("U0", "P0", "HH0")))
    if les:
        ch.upload_wall(np.asfortranarray(d["TAUW0"]), np.asfortranarray(d["TAUB0"]))
        ch.set_wsm(d["WSM0"])
    pg = pg3 = 0.0
    presg = []
    for n in range(1, int(d["steps"]) + 1):
        pg, pg3 = ch.step(n, dt, pg, pg3)
        presg.append(pg)
    return d, g, ch, presg


@pytest.mark.parametrize("fname,name,over,les", CASES)
def test_fp64_matches_reference_fixture(libc3d, fname, name, over, les):
    d, g, ch, presg = run(libc3d, fname, name, over, les, C3D_FP64)
    U, P, HH = ch.download()
    a, b = interior(g, U, P, HH), interior(g, d["U"], d["P"], d["HH"])
    for f in ("u", "v", "w", "hh", "p"):
        assert rel(a[f], b[f]) < 1e-10, (fname, f, rel(a[f], b[f]))
    np.testing.assert_allclose(presg, d["PRESG"][:, 0], rtol=1e-8)
    dg = ch.diagnose()
    assert abs(dg["divmax"] - float(d["DIVMAX"])) < 1e-13
    assert dg["cflm"] == pytest.approx(float(d["CFLM"]), rel=1e-12)
    assert dg["flow1"] == pytest.approx(float(d["FLOW"][0]), rel=1e-12)
    if les:
        S = ch.download_sgsvis()
        sl = (slice(1, g.n1m + 1), slice(None), slice(1, g.n3m + 1))
        assert rel(S[sl], d["SGSVIS"][sl]) < 1e-10
        tw, tb = ch.download_wall()
        isl = (slice(1, g.n1m + 1), slice(1, g.n3m + 1), slice(None))
        assert rel(tw[isl], d["TAUW"][isl]) < 1e-10 and rel(tb[isl], d["TAUB"][isl]) < 1e-10
        assert ch.get_wsm()[0] == pytest.approx(float(d["WSM"][0]), rel=1e-10)
    else:
        np.testing.assert_allclose(dg["wsm"], d["WSS"], rtol=1e-11, atol=1e-18)
    ch.close()


@pytest.mark.parametrize("fname,name,over,les", CASES)
def test_mixed_near_reference_fixture(libc3d, fname, name, over, les):
    d, g, ch, _ = run(libc3d, fname, name, over, les, C3D_MIXED)
    U, P, HH = ch.download()
    a, b = interior(g, U, P, HH), interior(g, d["U"], d["P"], d["HH"])
    for f in ("u", "v", "w"):
        assert rel(a[f], b[f]) < 2e-5, (fname, f, rel(a[f], b[f]))
    ch.close()

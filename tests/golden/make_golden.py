"""Writes the golden fixtures of this directory from the reference's own Fortran routines.

The reference (compact3d.f) is translated to C by ``oracle/f77c.py`` and compiled with gcc
(``oracle/ref.py``; FFTW replaced by ``oracle/fftw_shim.c``), because no Fortran compiler
exists on either machine.  Each fixture holds the inputs of a short run (the seeded,
projected initial state and, for LES, the initial wall state) and what the reference's
GETUP (compact3d.f:879-960) leaves after each step, plus the diagnostics of the last
state (DIVCHECK, CFL, CHKMF, WALLSS).  Run from the repository root:

    python tests/golden/make_golden.py

Fixtures:
  tiny16_dns.npz   16 x 16 x 16 cells, DNS (FILES 0), three steps from the seeded
                   perturbed-laminar start
  les16_les.npz    16 x 16 x 16 cells of the les32cs domain (8pi x 2 x 3pi, uniform y),
                   SGSCS + WALLMODEL_INSTANT, three steps from the seeded log-law start
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import ref  # noqa: E402
from compact3d_gb300 import ic  # noqa: E402
from compact3d_gb300.grid import make_grid  # noqa: E402

STEPS = 3


def run(name, les: bool, **over):
    g, dt = make_grid(name, **over)
    orc = oracle.Oracle(g)     # only for the projection of the seeded start
    if les:
        U, P, HH = ic.loglaw(g, 2000.0)
    else:
        U, P, HH = ic.perturbed_laminar(g)
    orc.project(U)
    R = ref.RefChannel(g)
    out = dict(U0=U.copy(), P0=P.copy(), HH0=HH.copy(), dt=dt, steps=STEPS)
    S = g.zeros_s() if les else None
    if les:
        tw, tb, wsm = orc.get_wall()
        R.set_wall(tw, tb)
        R.set_wsm(wsm)
        out.update(TAUW0=tw, TAUB0=tb, WSM0=wsm)
    pg = pg3 = 0.0
    presg = []
    for n in range(1, STEPS + 1):
        pg, pg3 = R.getup(U, P, HH, n, dt, pg, pg3, S)
        presg.append((pg, pg3))
    out.update(U=U, P=P, HH=HH, PRESG=np.array(presg))
    if les:
        tw, tb, wsm = R.get_wall()
        out.update(SGSVIS=S, TAUW=tw, TAUB=tb, WSM=wsm)
    out.update(DIVMAX=R.divcheck(U), CFLM=R.cfl(U), FLOW=np.array(R.chkmf(U)), WSS=R.wallss(U, P))
    return out


def main():
    for name, les, fname, over in (("tiny16", False, "tiny16_dns.npz", {}),
                                   ("les32cs", True, "les16_les.npz", dict(n1m=16, n3m=16))):
        d = run(name, les, **over)
        np.savez_compressed(os.path.join(HERE, fname), **d)
        print(fname, os.path.getsize(os.path.join(HERE, fname)), "bytes")


if __name__ == "__main__":
    main()

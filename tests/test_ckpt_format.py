"""The checkpoint format on the CPU: record layout, CWRITE's loop order, markers."""
import struct

import numpy as np

import ckpt_format as F
from compact3d_gb300 import ic
from compact3d_gb300.grid import make_grid


def test_records_follow_cwrite_order():
    g, _ = make_grid("small32")
    n1, n2m, n3 = g.n1m, g.n2m, g.n3m
    U, P, HH = ic.perturbed_laminar(g)
    data = F.records(n1, n2m, n3, 0.5, -0.25, 17, 3.5, U, P, HH)
    recs = F.split(data)
    assert len(recs) == 7
    assert struct.unpack("<3i", recs[0]) == (n1, n2m, n3)
    assert struct.unpack("<2d", recs[1]) == (0.5, -0.25)
    assert struct.unpack("<i", recs[2]) == (17,)
    assert struct.unpack("<d", recs[3]) == (3.5,)
    u = np.frombuffer(recs[4], "<f8")
    assert u.size == 3 * n1 * (n2m + 2) * n3
    # element (I, J, K, comp) of CWRITE's DO K / DO J=0,N2 / DO I loop with the three
    # components on one line
    for (I, J, K, c) in ((1, 0, 1, 0), (n1, n2m + 1, n3, 2), (5, 7, 11, 1)):
        pos = (((K - 1) * (n2m + 2) + J) * n1 + (I - 1)) * 3 + c
        assert u[pos] == U[I, J, K, c]
    p = np.frombuffer(recs[5], "<f8")
    I, J, K = 3, 4, 9
    assert p[((K - 1) * n2m + (J - 1)) * n1 + (I - 1)] == P[I - 1, J - 1, K - 1]
    h = np.frombuffer(recs[6], "<f8")
    nf = n1 * n2m * n3
    assert h[2 * nf + ((K - 1) * n2m + (J - 1)) * n1 + (I - 1)] == HH[I, J, K, 2]


def test_wall_record_with_sgs_model():
    g, _ = make_grid("les32cs")
    U, P, HH = ic.loglaw(g, 2000.0)
    tw = np.arange((g.n1m + 2) * (g.n3m + 2) * 2, dtype=float).reshape((g.n1m + 2, g.n3m + 2, 2), order="F")
    recs = F.split(F.records(g.n1m, g.n2m, g.n3m, 0, 0, 1, 0.0, U, P, HH, wall=(tw, -tw, [1.0, 2.0, 3.0])))
    assert len(recs) == 8
    w = np.frombuffer(recs[7], "<f8")
    assert w.size == 2 * tw.size + 3 and w[1] == tw.ravel(order="F")[1] and list(w[-3:]) == [1.0, 2.0, 3.0]

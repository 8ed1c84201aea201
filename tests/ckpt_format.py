"""The checkpoint format of c3d_checkpoint_write / c3d_checkpoint_read restated in numpy
(test infrastructure): Fortran sequential unformatted records with 4-byte little-endian
length markers, CWRITE's content and loop order (compact3d.f:832-872) plus the grid
extents, the AB2 history and, with an SGS model, the wall state."""
import struct

import numpy as np


def _rec(b: bytes) -> bytes:
    m = struct.pack("<i", len(b))
    return m + b + m


def records(n1, n2m, n3, presg, presg3, ntime, time, U, P, HH, wall=None):
    """Bytes of a checkpoint of the Fortran arrays U(0:M1,0:M2,0:M3,3), P(M1,M2,M3),
    HH(0:M1,0:M2,0:M3,3); wall = (TAUW, TAUB, WSM) with an SGS model."""
    n2 = n2m + 1
    out = [_rec(struct.pack("<3i", n1, n2m, n3)), _rec(struct.pack("<2d", presg, presg3)),
           _rec(struct.pack("<i", ntime)), _rec(struct.pack("<d", time))]
    u = np.asarray(U)[1:n1 + 1, 0:n2 + 1, 1:n3 + 1, :].transpose(2, 1, 0, 3)   # (K, J, I, comp)
    out.append(_rec(np.ascontiguousarray(u, dtype="<f8").tobytes()))
    p = np.asarray(P)[:n1, :n2m, :n3].transpose(2, 1, 0)
    out.append(_rec(np.ascontiguousarray(p, dtype="<f8").tobytes()))
    h = np.asarray(HH)[1:n1 + 1, 1:n2m + 1, 1:n3 + 1, :].transpose(3, 2, 1, 0)   # (NV, K, J, I)
    out.append(_rec(np.ascontiguousarray(h, dtype="<f8").tobytes()))
    if wall is not None:
        tw, tb, wsm = wall
        w = np.concatenate([np.asarray(tw).ravel(order="F"), np.asarray(tb).ravel(order="F"),
                            np.asarray(wsm, dtype=np.float64).ravel()])
        out.append(_rec(w.astype("<f8").tobytes()))
    return b"".join(out)


def split(data: bytes):
    """The records of a checkpoint file as a list of byte strings (markers checked)."""
    recs, pos = [], 0
    while pos < len(data):
        (m0,) = struct.unpack_from("<i", data, pos)
        body = data[pos + 4:pos + 4 + m0]
        (m1,) = struct.unpack_from("<i", data, pos + 4 + m0)
        assert m0 == m1 and len(body) == m0
        recs.append(body)
        pos += m0 + 8
    return recs

"""CPU checks of index maps that the CUDA kernels rely on.

* The four-step z FFT (k_fftz4, c3d_spec.cu): lane l holds frequencies k + N1 bitrev5(l)
  (k < N1) after its shuffle stages and writes them to tile row l + 32 k; the copy-out
  reads frequency q from row bitrev5(q / N1) + 32 (q mod N1).  The two maps must be
  inverse bijections of the 32 N1 rows, and the write must put the 16 lanes of each
  half-warp on 16 distinct bank pairs (8-byte elements, a tile pitch of 17 elements).
* The x passes in row segments of W lanes (c3d_xrows.cuh): the 32/W rows of a warp take
  J-dependent branches that hold shuffles, so for every shape the segment rule admits
  (rows of 48, 64, 96 points in 8 lanes, 128 in 16, N3M a multiple of 32/W) the rows of
  each warp must share J, for the block sizes the launchers use.
"""
import pytest


def bitrev5(v):
    return int(f"{v:05b}"[::-1], 2)


def bank_pair(row, col, pitch=17):
    return (row * pitch + col) % 16   # 8-byte elements: 16 bank pairs of 32 4-byte banks


@pytest.mark.parametrize("n1", [2, 3, 4, 6, 8, 12, 16])
def test_fftz_tile_rows_are_inverse_maps(n1):
    n = 32 * n1
    write = {}
    for lane in range(32):
        for k in range(n1):
            write[k + n1 * bitrev5(lane)] = lane + 32 * k
    assert sorted(write) == list(range(n)) and sorted(write.values()) == list(range(n))
    for q in range(n):
        assert write[q] == bitrev5(q // n1) + 32 * (q % n1)


@pytest.mark.parametrize("n1", [2, 3, 4, 6, 8, 12, 16])
def test_fftz_tile_write_is_conflict_free(n1):
    for k in range(n1):
        for c in range(16):
            for half in (range(16), range(16, 32)):
                assert len({bank_pair(lane + 32 * k, c) for lane in half}) == 16
    if n1 == 12:   # the frequency-row write it replaced: two bank pairs per half-warp (8-way)
        pairs = {bank_pair(0 + n1 * bitrev5(lane), 0) for lane in range(16)}
        assert len(pairs) == 2


def segment_lanes(n1m, n3m):
    """The segment rule of x_segment_lanes (c3d_xbatch.cu)."""
    w = 8 if n1m in (48, 64, 96) else 16 if n1m == 128 else 32
    return w if w < 32 and n3m % (32 // w) == 0 else 0


@pytest.mark.parametrize("n1m", [48, 64, 96, 128])
@pytest.mark.parametrize("n2m", [32, 48, 64, 96])
@pytest.mark.parametrize("n3m", [48, 64, 96, 128])
@pytest.mark.parametrize("xw", [2, 4, 8])
def test_row_segments_of_a_warp_share_j(n1m, n2m, n3m, xw):
    w = segment_lanes(n1m, n3m)
    assert w in (8, 16)
    nrows, rpb, per_warp = n2m * n3m, xw * 32 // w, 32 // w
    nblocks = -(-nrows // rpb)
    for blk in range(nblocks):
        for warp in range(xw):
            rows = [blk * rpb + warp * per_warp + s for s in range(per_warp)]
            live = [r < nrows for r in rows]
            assert all(live) or not any(live)          # a warp is whole or idle
            if all(live):
                assert len({1 + r // n3m for r in rows}) == 1

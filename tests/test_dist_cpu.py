"""The multi-GPU plumbing of bench.py on CPU: two gloo ranks on 127.0.0.1.

Single channels run as independent replicas, one per rank, with no collective on the
data path; the bench takes the maximum of the ranks' times and the sum of their points.
This checks those reductions and the barrier with world_size 2.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import importlib.util
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    D = bench.Dist()
    D.barrier()
    t = 1.5 + rank            # this rank's "time"
    pts = 1000 * (rank + 1)   # this rank's points
    out[rank] = (D.max(t), D.sum(pts), D.world, D.rank)
    D.barrier()
    D.close()


def test_two_rank_max_and_sum():
    port = _free_port()
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        tmax, psum, w, rk = res[r]
        assert tmax == 2.5 and psum == 3000 and w == 2 and rk == r

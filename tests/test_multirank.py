"""The N > 1 path of bench.py on CPU: replicas only, so the ranks exchange nothing but
the timing aggregate (updates summed, time = the slowest rank).  Two gloo ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import bench
    d = bench.Dist()
    d.barrier()
    upd = 1000 * (rank + 1)
    secs = 0.5 + rank
    out[rank] = (d.reduce(upd, "sum"), d.reduce(secs, "max"), d.local, d.world)
    d.close()


@pytest.mark.timeout(120)
def test_two_ranks_aggregate():
    world = 2
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        tot, mx, local, w = res[r]
        assert tot == 3000 and mx == 1.5 and local == r and w == 2


def test_single_rank_is_identity():
    import bench
    d = bench.Dist()
    assert d.world == 1 and d.reduce(7.0, "sum") == 7.0 and d.reduce(3.0, "max") == 3.0

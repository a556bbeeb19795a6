"""The N > 1 path of bench.py is replicas: every rank runs its own
propagation, the ranks meet at a barrier around the timed region, and the
slowest rank's time is the job's (max over ranks). Checked with two gloo
ranks on the CPU."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    r, w = bench.dist_init()
    bench.barrier(w)
    t = bench.allmax(1.0 + 2.5 * r, w)        # rank-dependent "elapsed time"
    bench.barrier(w)
    out[r] = (r, w, t)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for r, (rr, w, t) in res.items():
        assert rr == r and w == world
        assert t == 3.5                        # max over ranks of 1.0 + 2.5 r

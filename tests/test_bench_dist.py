"""CPU test (world size 2, gloo) of bench.py's multi-GPU logic: one independent shard per rank (no data-path
collective), the timing of the slowest rank, and the whole-job rate = units of all ranks / that time."""
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench
    import sid_gb300 as sid
    dist, r, w, local = bench.dist_setup("gloo")
    root = np.array([[0.295, 1.264912], [0.0, 1.264912], [0.0, 1.264912]])
    lo, hi = sid.synthetic_batch(root, 1000, seed=bench.shard_seed(r))
    local_seconds = 1.0 + r                       # the second rank is slower
    slowest = bench.max_over_ranks(dist, local_seconds, device="cpu")
    rate = bench.whole_job_rate(1000, w, slowest)
    out[r] = (float(lo.sum()), slowest, rate)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_independently_and_report_the_slowest():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] != res[1][0]                 # different shards
    assert res[0][1] == res[1][1] == 2.0          # both see the slowest rank's time
    assert res[0][2] == res[1][2] == 1000 * 2 / 2.0

"""CPU test (world size 2, gloo) of a sharded proof across ranks: each rank proves its part of the root
partition (the sid_prove_opts part_index/part_count contract, restated by the oracle), the only exchange is
one sum of the counters, and the sum equals the reference's published counts."""
import json
import os
import socket
import sys

import torch
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, name, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    sys.path.insert(0, os.path.join(REPO, "squares-in-disk_gb300", "python"))
    import torch.distributed as dist
    import oracle_py
    import sid_gb300 as sid
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r = oracle_py.prove(sid.lemma_ir(name), part=(rank, world), threads=2)
    counts = torch.tensor([r["cuboids"], r["leaves"], r["criticals"]], dtype=torch.int64)
    mine = counts.clone()
    dist.all_reduce(counts)
    out[rank] = (mine.tolist(), counts.tolist())
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_prove_their_shards_and_sum_to_the_published_counts():
    world, port, name = 2, _free_port(), "one_subcontainer"
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, name, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][1] == res[1][1] == PUBLISHED[name] + [0]
    assert res[0][0] != res[1][0] and all(c > 0 for c in res[0][0][:2] + res[1][0][:2])

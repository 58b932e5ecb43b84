"""GPU test of a sharded proof across processes: two ranks (gloo, world size 2), each with its own engine on
cuda:0, prove their parts of the root partition (sid_prove_opts part_index/part_count) and exchange only one
sum of the counters; the sum equals the reference's published counts. This is the engine-side form of
tests/test_shard_dist.py. Both ranks' kernels run independently on the one GPU (neither waits on the other);
on a multi-GPU node each rank would take its own device."""
import json
import os
import socket
import sys

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, name, precision, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, os.path.join(REPO, "squares-in-disk_gb300", "python"))
    import torch.distributed as dist
    import sid_gb300 as sid
    dist.init_process_group("gloo", rank=rank, world_size=world)
    eng = sid.Engine(0)
    r = eng.prove(eng.register(sid.lemma_ir(name)), precision=precision, part=(rank, world))
    eng.close()
    counts = torch.tensor([r["cuboids"], r["leaves"], r["criticals"]], dtype=torch.int64)
    mine = counts.clone()
    dist.all_reduce(counts)
    out[rank] = (mine.tolist(), counts.tolist())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("name,precision", [("one_subcontainer", 0), ("three_subcontainer", 1)])
def test_two_processes_prove_their_shards_and_sum_to_the_published_counts(name, precision):
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(world, port, name, precision, out), nprocs=world, join=True,
                           start_method="spawn")
        res = dict(out)
    assert res[0][1] == res[1][1] == PUBLISHED[name] + [0]
    assert res[0][0] != res[1][0] and all(c > 0 for c in res[0][0][:2] + res[1][0][:2])

"""The N > 1 host path of bench.py on CPU (gloo, world size 2): each rank is
an independent replica with its own parameter sets, and the job's step time
and units are the max and the sum over the ranks.  No collective touches the
data path; these are the only two reductions."""
import os
import socket
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        w = bench.workload("batched512", rank)
        sets = [None] * world
        dist.all_gather_object(sets, w["sets"])
        ms, units = bench.reduce_across_ranks(1.0 + rank, 10.0 * (rank + 1), "cpu")
        out.put((rank, sets, ms, units, bench.total_radii(w)))
    finally:
        dist.destroy_process_group()


def test_replicas_distinct_sets_and_reductions():
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, sets, ms, units, nr in res:
        assert ms == 2.0            # max of 1.0, 2.0
        assert units == 30.0        # 10 + 20
        assert len(sets[0]) == len(sets[1]) == 64
        assert sets[0] != sets[1]   # each replica has its own parameter sets
        assert nr > 64
    # a rank's own workload is reproducible and rank 0 is the single-GPU one
    sys.path.insert(0, ROOT)
    import bench
    assert bench.workload("batched512", 0)["sets"] == res[0][1][0]
    assert bench.workload("batched512")["sets"] == res[0][1][0]

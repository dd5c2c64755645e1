"""Replicas-only multi-process path of bench.py on CPU: world size 2 over gloo, each rank times
its own replica and the job time is the max over ranks."""
import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(1.0 + rank, None)
    bench.barrier()
    # each rank advances its own replica through the oracle (host path) and reports a checksum
    from oracle.pyoracle import Oracle
    from plens_gb300 import configs
    case = configs.make_case(configs.sod(n=8))
    o = Oracle(case, threads=1)
    o.set_state(case.initial_state(), 0.0)
    o.advance(2)
    U = o.get_state()[0]
    q.put((rank, t, float(U.sum())))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_replicas_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=100) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[1] for r in res] == [2.0, 2.0]          # max over ranks seen by every rank
    assert res[0][2] == res[1][2]                     # identical replicas

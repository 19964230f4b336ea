"""Multi-rank logic of the benchmark on CPU: two gloo ranks (127.0.0.1).
Multi-GPU runs are independent replicas (each rank builds its own molecule or
batch, no collective on the data path); the only collective is the
max-over-ranks of the timed region and the barrier around it."""
import os
import socket

import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ws, r, local = bench.dist_env()
    dist.barrier()
    m = bench.max_over_ranks(1.5 + r)
    # replicas: each rank seeds its own batch of molecules
    from openqp_gb300 import workloads
    sizes = list(workloads.np.random.default_rng(0 + r).integers(1, 17, 8))
    q.put((r, ws, local, m, sizes))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_replica_seeds():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [2, 2]
    assert [o[0] for o in out] == [0, 1] and [o[2] for o in out] == [0, 1]
    assert all(o[3] == 2.5 for o in out)
    assert out[0][4] != out[1][4]


def test_single_rank_max_is_identity():
    import bench
    assert bench.max_over_ranks(3.25) == 3.25

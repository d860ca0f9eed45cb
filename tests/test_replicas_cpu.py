"""Multi-GPU runs of this path are replicas only (a single cloth does not shard
without a halo exchange every sweep): each rank steps its own copy, the job
time is the slowest rank's.  The rank-level logic of bench.py is exercised
here with world size 2 on the gloo backend, on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    d = bench.init_dist(world, "gloo")
    ws, r, local = bench.dist_env()
    bench.barrier(d)
    t = bench.max_over_ranks(d, 100.0 * (rank + 1))      # rank 1 is the slow one
    v = bench.aggregate_steps_per_s(ws, 10, t)
    bench.barrier(d)
    d.destroy_process_group()
    q.put((r, ws, t, v))


def test_replicas_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    for r, ws, t, v in res:
        assert ws == 2 and t == 200.0
        assert abs(v - 2 * 10 / 0.2) < 1e-9       # both replicas' steps over the slowest rank's time

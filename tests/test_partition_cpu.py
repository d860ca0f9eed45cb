"""Batched independent instances (config 2: cloths with their own obstacles)
partitioned across ranks by cumulative vertex count (pdipc_partition_instances,
host only), one process per GPU with no exchange in the step.

The planner is checked on its own, then with world size 2 on the gloo backend
on the CPU: each rank steps its slice of a small batch on the oracle, the
slices are gathered on rank 0 and compared with one single-rank run of the
whole batch.  Before any contact the instances share nothing (the stopping
rule is fixed to 2 outer iterations, so no global residual couples them
either), so the slices must reproduce the whole run bit for bit.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_partition_balances_cumulative_vertex_counts(built_lib):
    import pdipc
    sizes = np.array([100, 100, 100, 100], np.int64)
    assert list(pdipc.partition_instances(sizes, 2)) == [0, 2, 4]
    assert list(pdipc.partition_instances(sizes, 4)) == [0, 1, 2, 3, 4]
    assert list(pdipc.partition_instances(sizes, 1)) == [0, 4]
    uneven = np.array([900, 50, 50, 50, 50, 900], np.int64)
    f = pdipc.partition_instances(uneven, 2)
    assert list(f) == [0, 3, 6]                     # 1000 | 1000
    f = pdipc.partition_instances(np.array([5, 7], np.int64), 4)  # more ranks than instances
    assert f[0] == 0 and f[-1] == 2 and np.all(np.diff(f) >= 0)
    from pdipc import scenes
    sc = scenes.batched(256, 16, 128, seed=0, steps=1)
    sz = np.array([c.X.shape[0] for c in sc.cloths], np.int64)
    for ranks in (2, 4, 8):
        f = pdipc.partition_instances(sz, ranks)
        loads = np.add.reduceat(sz, f[:-1])
        assert f[0] == 0 and f[-1] == 256 and np.all(np.diff(f) > 0)
        assert loads.max() - loads.min() <= sz.max()   # within one instance of even


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _batch():
    from pdipc import scenes
    return scenes.batched(5, 6, 12, seed=4, steps=3)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import pdipc
    from oracle.oracle import FORM_JJ, Oracle
    from pdipc import scenes
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo")
    sc = _batch()
    sizes = np.array([c.X.shape[0] for c in sc.cloths], np.int64)
    first = pdipc.partition_instances(sizes, world)
    mine = scenes.instance_slice(sc, int(first[rank]), int(first[rank + 1]))
    orc = Oracle(mine, "fp64", FORM_JJ, threads=1, fixed_outer=2)
    orc.step(3)
    x = torch.from_numpy(np.ascontiguousarray(orc.positions()[:mine.n_sim]))
    n = torch.tensor([x.shape[0]])
    ns = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(ns, n)
    width = int(max(int(v) for v in ns))
    pad = torch.zeros((width, 3), dtype=torch.float64)
    pad[:x.shape[0]] = x
    bufs = [torch.zeros((width, 3), dtype=torch.float64) for _ in range(world)]
    dist.all_gather(bufs, pad)
    dist.destroy_process_group()
    if rank == 0:
        q.put(np.concatenate([b[:int(k)].numpy() for b, k in zip(bufs, ns)]))
    else:
        q.put(None)


def test_partitioned_batch_matches_single_rank_run_gloo(built_lib):
    import torch.multiprocessing as mp
    from oracle.oracle import FORM_JJ, Oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = [q.get(timeout=300) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    gathered = next(g for g in got if g is not None)
    sc = _batch()
    whole = Oracle(sc, "fp64", FORM_JJ, threads=1, fixed_outer=2)
    whole.step(3)
    assert whole.stats()["active_contacts"] == 0
    ref = whole.positions()[:sc.n_sim]
    assert gathered.shape == ref.shape
    assert np.array_equal(gathered, ref)

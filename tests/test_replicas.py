"""Multi-GPU replicas, host side: unit sharding and the result gather, run
as two gloo ranks on the CPU (each rank "solves" its units with the CPU
oracle on tiny grids, the work a GPU rank would do with the solver)."""
import os
import socket

import numpy as np
import pytest

from poe2d_gb300.replicas import shard


def test_shard_is_a_balanced_partition():
    rng = np.random.default_rng(0)
    costs = list(rng.integers(256, 1537, 37) ** 3 * 4)
    for world in (1, 2, 3, 8):
        parts = shard(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        lower = max(max(costs), sum(costs) / world)          # no schedule beats this
        assert max(loads) <= 4.0 / 3.0 * lower + 1e-9
    assert shard(costs, 2) == shard(costs, 2)                 # deterministic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    from oracle import oracle as O
    from poe2d_gb300.replicas import gather, max_over_ranks, shard as sh
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = [24, 31, 17, 40, 28]
    mine = sh([n ** 3 for n in sizes], world)[rank]
    res = {}
    for i in mine:
        n = sizes[i]
        coef = np.zeros((8, n + 1, n + 1), np.float32)
        coef[0], coef[1], coef[2], coef[3] = 2320.0, 1000.0, 1e4, 1e9
        coef[4], coef[5], coef[6], coef[7] = 9.8e9, 8e9, 0.73, 9.7e9
        px = np.zeros((6, n + 1), np.float32)
        pz = np.zeros((6, n + 1), np.float32)
        px[1], px[2], px[4], px[5] = 1, 1, 1, 1
        pz[1], pz[2], pz[4], pz[5] = 1, 1, 1, 1
        o = O.Oracle(O.F32, n, n, 0.5, 0.5, 5e-5, coef, px, pz, threads=1)
        o.set_source(n // 2, n // 2, O.SRC_FZ, O.source_table(1, 200.0, 5e-5, 20, amplitude=1e3, t_cut=0.0,
                                                              dx=0.5, dz=0.5))
        o.set_receivers([(n // 2, n // 2 - 3, 1)])
        res[i] = float(np.abs(o.run(20)).sum())
    merged = gather(res)
    t = max_over_ranks(float(rank + 1))
    if rank == 0:
        q.put((sorted(merged), merged, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_gather():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    keys, merged, t = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert keys == [0, 1, 2, 3, 4]
    assert all(v > 0 for v in merged.values())
    assert t == 2.0

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


def _oracle_solve(specs):
    """What gpu_solve does on a GPU, on the CPU oracle: each spec's model
    (datagen.build_model with a thin C-PML and 8 receivers) for its steps."""
    from oracle import oracle as O
    from poe2d_gb300 import datagen as D
    out = {}
    for sp in specs:
        g, coef, px, pz, src, rec, _ = D.build_model(sp, npml=4, nrec=8)
        o = O.Oracle(O.F32, g.NX, g.NZ, g.dx, g.dz, g.dt, coef, px, pz, threads=1)
        o.set_source(src.ix, src.iz, O.SRC_FZ, O.source_table(1, src.f0, g.dt, sp["steps"], amplitude=src.amplitude,
                                                              t_cut=0.0, dx=g.dx, dz=g.dz))
        o.set_receivers(rec)
        out[sp["index"]] = o.run(sp["steps"])
    return out


def _runner_rank(rank, world, port, q):
    import torch.distributed as dist
    from poe2d_gb300 import batch_runner as BR
    from poe2d_gb300 import datagen as D
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = D.uneven_specs(3, 7, n_min=24, n_max=44)
    mine = shard([BR.cost(sp) for sp in specs], world)[rank]
    merged, el = BR.run(specs, _oracle_solve)
    q.put((rank, mine, None if merged is None else {k: v.tolist() for k, v in merged.items()}, el))
    dist.destroy_process_group()


def test_batch_runner_shards_models_over_two_ranks():
    """The uneven-batch runner on two gloo ranks: every model is solved by
    exactly one rank (the LPT shard), rank 0 receives every model's traces
    and they equal a one-process run of the same models."""
    import torch.multiprocessing as mp
    from poe2d_gb300 import datagen as D
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_runner_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=240) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by_rank = {r: (mine, merged, el) for r, mine, merged, el in got}
    assert sorted(by_rank[0][0] + by_rank[1][0]) == list(range(7)) and by_rank[0][0] and by_rank[1][0]
    assert by_rank[1][1] is None and by_rank[0][2] == by_rank[1][2] > 0     # the slowest rank's time on both
    merged = by_rank[0][1]
    specs = D.uneven_specs(3, 7, n_min=24, n_max=44)
    want = _oracle_solve(specs)
    assert sorted(merged) == list(range(7))
    for k, v in want.items():
        assert np.array_equal(np.asarray(merged[k], np.float32), v), k
        assert np.abs(v).max() > 0

"""Uneven batches over several GPUs: one process per GPU, each running its
share of the models as batches on its own GPU, rank 0 collecting the gathers.

The reference runs one shot of one model per process (its shot loop and the
commented shift of the source between shots, cu:1615 and cu:1732-1735).
Here the models of a batch (patchy realisations of uneven sizes and step
counts, ``datagen.uneven_specs``) are independent units: each rank takes the
models ``replicas.shard`` gives it (longest first to the least-loaded rank,
by cell-updates), advances them in groups of ``group`` models with the
batched solver (one launch per time step over every tile of every model of
the group), and the results meet on rank 0 in one gather after the work.
There is no collective on the data path.

    torchrun --nproc-per-node N -m poe2d_gb300.batch_runner --models 256 --out gathers.npz

``run(specs, solve, pg)`` is the rank-side driver; ``solve(specs)`` turns a
list of specs into ``{index: traces}``.  ``gpu_solve`` is the batched-solver
implementation (the default); any other function with that contract (a
different recording, a smaller resampled output) can be passed instead.
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

from . import replicas


def cost(spec):
    """Cell-updates of one model: side^2 cells x steps."""
    return float(spec["side"]) ** 2 * float(spec["steps"])


def gpu_solve(specs, group=64, fast=True, resample_to=None, stream=None):
    """Run specs on the current CUDA device in batches of `group` models:
    {index: traces (steps x receivers), or resampled to resample_to samples}."""
    from . import datagen as D
    from .solver import Batch, Solver
    out = {}
    for g0 in range(0, len(specs), group):
        part = specs[g0:g0 + group]
        solvers = []
        try:
            for sp in part:
                g, coef, px, pz, src, rec, _ = D.build_model(sp)
                s = Solver(g, coef, px, pz, stream=stream, fast=fast)
                s.add_shot(src, rec)
                solvers.append(s)
            with Batch(solvers, stream=stream) as b:
                b.run([sp["steps"] for sp in part])
                b.sync()
            for sp, s in zip(part, solvers):
                tr = s.traces(0)
                out[sp["index"]] = D.resample(tr, resample_to) if resample_to else tr
        finally:
            for s in solvers:
                s.close()
    return out


def run(specs, solve, pg=None):
    """This rank's share of specs through solve(); rank 0 returns every
    model's result ({index: value}) and the slowest rank's seconds, the other
    ranks (None, that time)."""
    import torch.distributed as dist
    world = dist.get_world_size(pg) if dist.is_initialized() else 1
    rank = dist.get_rank(pg) if dist.is_initialized() else 0
    mine = replicas.shard([cost(sp) for sp in specs], world)[rank]
    t0 = time.perf_counter()
    res = solve([specs[i] for i in mine])
    el = replicas.max_over_ranks(time.perf_counter() - t0, pg)
    return replicas.gather(res, pg), el


def main(argv=None):
    ap = argparse.ArgumentParser(description="uneven patchy batch over the GPUs of one node")
    ap.add_argument("--models", type=int, default=256)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--group", type=int, default=64, help="models per batched launch sequence")
    ap.add_argument("--resample", type=int, default=0, help="samples per trace (0: keep every step)")
    ap.add_argument("--exact", action="store_true", help="the reference's rounding instead of FP32 stencils")
    ap.add_argument("--out", default="", help="npz file written by rank 0")
    args = ap.parse_args(argv)
    import torch
    import torch.distributed as dist
    from . import datagen as D
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    specs = D.uneven_specs(args.seed, args.models)
    st = torch.cuda.Stream()
    merged, el = run(specs, lambda sp: gpu_solve(sp, args.group, not args.exact, args.resample or None,
                                                  st.cuda_stream))
    if merged is not None:
        work = sum(cost(sp) for sp in specs)
        print("%d models on %d GPU(s): %.1f s, %.1f Gcell-updates/s" % (len(merged), world, el, work / el / 1e9))
        if args.out:
            np.savez_compressed(args.out, **{"model_%05d" % k: v for k, v in sorted(merged.items())})
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

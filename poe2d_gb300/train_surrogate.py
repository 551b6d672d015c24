"""Train and evaluate the surrogate on gathers the batched solver generates.

    python -m poe2d_gb300.train_surrogate --train 2048 --heldout 256 --epochs 30

Pipeline (one GPU):
  1. data     uneven patchy models (poe2d_gb300.datagen: side U[256, 1536],
              steps 4 x side, porosity, gas fraction, patch radius, f0 drawn
              per model), one centre-surface shot each with 128 receivers x
              (vx, vz, p), advanced by the batched solver (Batch) in groups;
              traces resampled to 1024 samples, normalised per component by
              the training set's RMS, stored bf16 on the device.  Inputs: the
              gas-fraction map area-averaged to 64 x 64, a constant porosity
              channel, and (f0, side, porosity) as scalars.
  2. train    four networks from different seeds (the ensemble), Adam, batch
              64, lr 3e-4 with cosine decay, every kernel the library's own.
  3. evaluate held-out models never seen in training: the ensemble mean is
              accepted where the members agree within the threshold (5 %
              relative spread), otherwise the solver result is used; reports
              the relative L2 error of accepted gathers against the solver,
              the acceptance rate and gathers/s of the surrogate, of the
              solver alone and of surrogate + fallback.
Relative L2 errors are taken on the normalised gathers (each component
scaled by its training-set RMS, so vx, vz and p weigh alike).
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

SAMPLES, NREC, MAP = 1024, 128, 64


def _timed(stream, fn):
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    r = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return r, e0.elapsed_time(e1) * 1e-3


def model_inputs(spec, ids):
    """(map [64, 64, 2], scalars [3]) of one model."""
    n = ids.shape[0]
    edges = (np.arange(MAP + 1) * n) // MAP
    g = np.add.reduceat(np.add.reduceat(ids.astype(np.float32), edges[:-1], axis=0), edges[:-1], axis=1)
    area = np.outer(np.diff(edges), np.diff(edges)).astype(np.float32)
    gas = g / area
    phi = (spec["phi"] - 0.2) / 0.1
    m = np.stack([np.full((MAP, MAP), phi, np.float32), gas], axis=-1)
    sc = np.array([(spec["f0"] - 225.0) / 75.0, (spec["side"] - 896.0) / 640.0, phi], np.float32)
    return m, sc


def generate(specs, stream, group=64, fast=True):
    """Run the solver on every spec, `group` models per batch.  The host
    builds the next group's models while the GPU runs the current batch;
    groups alternate between two creation streams, because a batch orders
    its contexts' streams after itself.  Returns maps [N, 64, 64, 2] f32, scalars [N, 3],
    gathers [N, 1024, 384] f32 (host), the batches' device time in seconds
    and the cell-updates done."""
    import torch
    import poe2d_gb300 as P
    from poe2d_gb300 import datagen as D
    N = len(specs)
    maps = np.zeros((N, MAP, MAP, 2), np.float32)
    scal = np.zeros((N, 3), np.float32)
    gath = np.zeros((N, SAMPLES, 3 * NREC), np.float32)
    cstreams = [torch.cuda.Stream(), torch.cuda.Stream()]
    t_solver, cells = 0.0, 0

    def build(g0):
        cstream = cstreams[(g0 // group) % 2]
        solvers = []
        for i, sp in enumerate(specs[g0:g0 + group]):
            g, coef, px, pz, src, rec, ids = D.build_model(sp, nrec=NREC)
            maps[g0 + i], scal[g0 + i] = model_inputs(sp, ids)
            s = P.Solver(g, coef, px, pz, stream=cstream.cuda_stream, fast=fast)
            s.add_shot(src, rec)
            solvers.append(s)
        return solvers

    def finish(job):
        nonlocal t_solver
        g0, solvers, b, e0, e1 = job
        b.sync()
        e1.synchronize()
        t_solver += e0.elapsed_time(e1) * 1e-3
        b.close()
        for i, s in enumerate(solvers):
            gath[g0 + i] = D.resample(s.traces(0), SAMPLES)
            s.close()

    job = None
    for g0 in range(0, N, group):
        solvers = build(g0)
        cstreams[(g0 // group) % 2].synchronize()
        if job:
            finish(job)
        part = specs[g0:g0 + group]
        cells += sum(sp["side"] ** 2 * sp["steps"] for sp in part)
        b = P.Batch(solvers, stream=stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run([sp["steps"] for sp in part])
        e1.record(stream)
        job = (g0, solvers, b, e0, e1)
    if job:
        finish(job)
    return maps, scal, gath, t_solver, cells


def rel_err(pred, true):
    """Per-model relative L2 error of [N, ...] arrays."""
    d = (pred - true).reshape(pred.shape[0], -1)
    t = true.reshape(true.shape[0], -1)
    return np.linalg.norm(d, axis=1) / np.maximum(np.linalg.norm(t, axis=1), 1e-30)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2048)
    ap.add_argument("--heldout", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--members", type=int, default=4)
    ap.add_argument("--threshold", type=float, default=0.05)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--side-min", type=int, default=256)
    ap.add_argument("--side-max", type=int, default=1536)
    ap.add_argument("--gas-max", type=float, default=0.3, help="0: homogeneous (gas-free) models only")
    ap.add_argument("--phi", type=float, nargs=2, default=(0.1, 0.3))
    ap.add_argument("--f0", type=float, nargs=2, default=(150.0, 300.0))
    ap.add_argument("--out", default=None, help="write the summary JSON here")
    args = ap.parse_args(argv)

    import torch
    import poe2d_gb300 as P
    from poe2d_gb300 import datagen as D
    from poe2d_gb300.surrogate import Surrogate, gather_rows
    P.lib()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    t_all = time.perf_counter()

    # 1. data: training realisations and held-out realisations from other seeds
    spec_tr = []
    for k in range(math.ceil(args.train / 256)):
        spec_tr += D.uneven_specs(args.seed * 1000 + k, 256, args.side_min, args.side_max, args.gas_max, args.phi,
                                  args.f0)
    spec_tr = spec_tr[:args.train]
    spec_ho = []
    for k in range(math.ceil(args.heldout / 256)):      # seeds counting down from 999: none a training seed
        spec_ho += D.uneven_specs(args.seed * 1000 + 999 - k, 256, args.side_min, args.side_max, args.gas_max,
                                  args.phi, args.f0)
    spec_ho = spec_ho[:args.heldout]
    t0 = time.perf_counter()
    m_tr, s_tr, y_tr, ts_tr, c_tr = generate(spec_tr, stream)
    m_ho, s_ho, y_ho, ts_ho, c_ho = generate(spec_ho, stream)
    t_data = time.perf_counter() - t0
    rms = np.sqrt(np.mean(y_tr.reshape(len(spec_tr), SAMPLES, 3, NREC) ** 2, axis=(0, 1, 3)))   # per component
    scale = np.repeat(rms, NREC).astype(np.float32)                  # channel c = 128 * comp + receiver
    y_tr /= scale
    y_ho /= scale
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dtype=dt).cuda()
    Mtr, Str, Ytr = dev(m_tr, torch.bfloat16), dev(s_tr, torch.float32), dev(y_tr, torch.bfloat16)
    Mho, Sho = dev(m_ho, torch.bfloat16), dev(s_ho, torch.float32)
    del y_tr

    # 2. train the ensemble
    nb = len(spec_tr) // args.batch
    steps = nb * args.epochs
    members, curves, t_train = [], [], 0.0
    for k in range(args.members):
        net = Surrogate(max_batch=max(args.batch, 256), seed=1000 + k, stream=stream.cuda_stream)
        rng = np.random.default_rng(k)
        curve, it = [], 0
        t0 = time.perf_counter()
        for ep in range(args.epochs):
            perm = torch.from_numpy(rng.permutation(len(spec_tr))).cuda()
            tot = 0.0
            for bi in range(nb):
                idx = perm[bi * args.batch:(bi + 1) * args.batch]
                lr = args.lr * 0.5 * (1.0 + math.cos(math.pi * it / steps))
                tot += net.train_step(gather_rows(Mtr, idx), gather_rows(Str, idx), gather_rows(Ytr, idx), lr)
                it += 1
            curve.append(tot / nb)
        torch.cuda.synchronize()
        t_train += time.perf_counter() - t0
        curves.append(curve)
        members.append(net)

    # 3. held-out evaluation
    def infer():
        outs = []
        for net in members:
            o = torch.empty((len(spec_ho), SAMPLES, 3 * NREC), dtype=torch.float32, device="cuda")
            for b0 in range(0, len(spec_ho), 256):
                b1 = min(b0 + 256, len(spec_ho))
                net.forward(Mho[b0:b1], Sho[b0:b1], out=o[b0:b1])
            outs.append(o)
        return torch.stack(outs)
    infer()                                                   # warm-up
    preds, t_sur = _timed(stream, infer)
    P_ = preds.cpu().numpy()
    mean = P_.mean(axis=0)
    spread = np.max(np.stack([rel_err(P_[k], mean) for k in range(len(members))]), axis=0)
    err = rel_err(mean, y_ho)
    accept = spread <= args.threshold
    # fallback: the solver for the rejected models
    rej = [spec_ho[i] for i in np.nonzero(~accept)[0]]
    t_fb = 0.0
    if rej:
        _, _, _, t_fb, _ = generate(rej, stream)
    n = len(spec_ho)
    summary = {
        "family": {"side": [args.side_min, args.side_max], "gas_max": args.gas_max, "phi": list(args.phi),
                   "f0": list(args.f0)},
        "train_models": len(spec_tr), "heldout_models": n, "epochs": args.epochs, "batch": args.batch,
        "members": len(members), "params_per_member": members[0].nparam,
        "data_s": t_data, "solver_s_train": ts_tr, "solver_s_heldout": ts_ho,
        "solver_gcells": (c_tr + c_ho) / (ts_tr + ts_ho) / 1e9,
        "train_s": t_train, "train_steps_per_member": steps,
        "loss_first_last": [[c[0], c[-1]] for c in curves],
        "component_rms": rms.tolist(),
        "heldout_rel_l2_all": {"median": float(np.median(err)), "mean": float(err.mean()),
                               "p90": float(np.percentile(err, 90))},
        "threshold": args.threshold, "accepted": int(accept.sum()),
        "accepted_rel_l2": ({"median": float(np.median(err[accept])), "mean": float(err[accept].mean()),
                             "max": float(err[accept].max())} if accept.any() else None),
        "accepted_within_5pct": int(np.sum(err[accept] <= 0.05)) if accept.any() else 0,
        "spread_vs_error_corr": float(np.corrcoef(spread, err)[0, 1]) if n > 2 else None,
        "surrogate_gathers_per_s": n / t_sur, "solver_gathers_per_s": n / ts_ho,
        "surrogate_speedup_vs_solver": (n / t_sur) / (n / ts_ho),
        "with_fallback_gathers_per_s": n / (t_sur + t_fb), "fallback_s": t_fb,
        "with_fallback_speedup_vs_solver": (n / (t_sur + t_fb)) / (n / ts_ho),
        "wall_s": time.perf_counter() - t_all,
    }
    for net in members:
        net.close()
    line = json.dumps(summary)
    print(line, flush=True)
    if args.out:
        with open(args.out, "w") as f:
            f.write(line + "\n")
    return summary


if __name__ == "__main__":
    main()

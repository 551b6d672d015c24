"""Benchmark: the 2-D poroelastic C-PML time loop on GB300.

Workload (one bench step = one complete shot):
  2001 x 2001 patchy-saturation model, h = 0.5 m, 40-cell C-PML on all sides;
  sandstone frame (rho_s 2650, phi 0.2, K_s 37 GPa, K_frame 10 GPa,
  mu 8 GPa, kappa 1e-12, tortuosity 2), water background (K_f 2.25 GPa,
  rho_f 1000, eta 1e-3) with seeded random circular gas patches (K_gas
  0.02 GPa, rho_gas 100, eta 1e-5, radii U[2, 10] m, 10 % areal fraction);
  dt = 5e-5 s, 20000 steps; Ricker f0 = 200 Hz vertical force at the surface
  centre; 400 surface receivers recording vx, vz and p.
Inputs are synthetic (seeded), the reference ships no model files.

value: Gcell-updates/s with the model resident in HBM (state reset + 20000
steps per bench step, CUDA events around K steps).  e2e: the same through
the C ABI from pinned host buffers: create context (coefficients in, palette
built on the host, ids uploaded), run, read the traces back (D2H), destroy.
cpu_baseline / --impl reference: the CPU oracle (a C restatement of the
reference loop, OpenMP over all host threads) on a bounded sample of steps of
the same model.

batched (--batched M, default 64; 0 skips): the metric's "batched vs 1-shot"
part.  (a) 64 shots of one 1001 x 1001 patchy model (30-cell C-PML, 10000
steps, 256 receivers x 3 per shot) in one launch per step, against the same
shots run one at a time; (b) M of the 256 uneven models (side U[256, 1536],
steps 4 x side) in one batch, against back-to-back single-model runs.  Both
check that the batched traces equal the single runs bit for bit.
surrogate: gathers/s of the 4-member ensemble's forward passes at batch 256
on the tensor cores, beside the batched solver's gathers/s on (b); and the
whole learned pipeline (solver gathers -> training -> held-out scoring with
solver fallback) on the narrow family the network learns
(--no-surrogate-train skips it).

Multi-GPU: shots are independent, so N ranks run N replicas (one shot each,
sources shifted), with no collective on the data path ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched Gcell-updates/s vs 1-shot at 1e-5; surrogate gathers/s at ≤5% L2 err"
NX = NZ = 2000
DX, DT, F0, NPML, NSTEPS, NREC = 0.5, 5e-5, 200.0, 40, 20000, 400


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


FRAME = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
WATER = dict(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **FRAME)
GAS = dict(rho_f=100.0, k_f=0.02e9, eta=1e-5, **FRAME)


def workload(seed=0, shift=0, via="product"):
    """The benchmark shot.  via="product": coefficients and C-PML profiles
    from the library; via="oracle": from the oracle's restatements (bit for
    bit the same arrays), so the CPU reference arm never loads the library."""
    import poe2d_gb300 as P
    from poe2d_gb300.patchy import random_patches
    ids = random_patches((NZ + 1, NX + 1), DX, fraction=0.10, r_min=2.0, r_max=10.0, seed=1234 + seed)
    g = P.grid(NX, NZ, DX, DT)
    if via == "oracle":
        from oracle import oracle as O
        coef, vp = O.coeffs_biot([WATER, GAS], ids)
        px, pz = O.pml_profiles(NX, NZ, DX, DX, DT, NPML, vp, f0=F0)
    else:
        coef, vp = P.coeffs_biot([P.biot_material(**WATER), P.biot_material(**GAS)], ids)
        P.check_courant(g, vp)
        px, pz = P.pml_profiles(g, NPML, F0, vp)
    isrc = (NX + 1) // 2 + shift
    src = P.source(isrc, NPML, P.SRC_RICKER_FZ, F0, 1e6, 0.0)
    xs = NPML + 1 + (np.arange(NREC) * (NX - 2 * NPML - 2)) // (NREC - 1)
    rec = [(int(x), NPML, c) for c in (P.REC_VX, P.REC_VZ, P.REC_P) for x in xs]
    return g, coef, px, pz, src, rec, ids


def shots_model(nshots=64, n=1001, npml=30, nrec=256):
    """The batched-shots workload: one n x n patchy model (the statistics of
    the single-shot model, 30-cell C-PML), nshots Ricker sources spaced evenly
    along the surface row, nrec surface receivers x (vx, vz, p) per shot."""
    import poe2d_gb300 as P
    from poe2d_gb300.patchy import random_patches
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = P.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    gas = P.biot_material(rho_f=100.0, k_f=0.02e9, eta=1e-5, **frame)
    ids = random_patches((n, n), DX, fraction=0.10, r_min=2.0, r_max=10.0, seed=4321)
    coef, vp = P.coeffs_biot([water, gas], ids)
    g = P.grid(n - 1, n - 1, DX, DT)
    P.check_courant(g, vp)
    px, pz = P.pml_profiles(g, npml, F0, vp)
    span = n - 1 - 2 * npml - 2
    srcs = [P.source(int(npml + 1 + (k * span) // max(nshots - 1, 1)), npml, P.SRC_RICKER_FZ, F0, 1e6, 0.0)
            for k in range(nshots)]
    xs = npml + 1 + (np.arange(nrec) * span) // (nrec - 1)
    rec = [(int(x), npml, c) for c in (P.REC_VX, P.REC_VZ, P.REC_P) for x in xs]
    return g, coef, px, pz, srcs, rec


def timed(stream, fn):
    """CUDA-event time (s) of fn() on stream, synchronised on both sides."""
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) * 1e-3


def leg_shots(P, stream, fast, nsteps=10000, nshots=64, single_shots=2):
    """64 shots of one model advanced together (one persistent launch per
    time step over every tile of every shot) against the same shots run one at
    a time; the batched traces of shot 0 must equal its single run's bit for bit."""
    g, coef, px, pz, srcs, rec = shots_model(nshots)
    cells = (g.NX + 1) * (g.NZ + 1)
    sb = P.Solver(g, coef, px, pz, stream=stream.cuda_stream, fast=fast)
    for s in srcs:
        sb.add_shot(s, rec)
    sb.run(64)                                   # warm-up: graph capture, first touch
    for k in range(nshots):
        sb.reset_shot(k)
    t_b = timed(stream, lambda: sb.run(nsteps))
    tr_b = sb.traces(0)
    sb.close()
    s1 = P.Solver(g, coef, px, pz, stream=stream.cuda_stream, fast=fast)
    s1.add_shot(srcs[0], rec)
    s1.run(64)
    s1.reset_shot(0)

    def singles():
        for _ in range(single_shots):
            s1.reset_shot(0)
            s1.run(nsteps)
    t_1 = timed(stream, singles) / single_shots
    same = bool(np.array_equal(s1.traces(0).view(np.uint32), tr_b.view(np.uint32)))
    s1.close()
    vb = cells * nsteps * nshots / t_b / 1e9
    v1 = cells * nsteps / t_1 / 1e9
    return {"workload": "%d shots x %dx%d patchy model, 30-cell C-PML, %d steps, %d receivers x (vx,vz,p) per shot"
                        % (nshots, g.NX + 1, g.NZ + 1, nsteps, len(rec) // 3),
            "batched_gcells": vb, "single_shot_gcells": v1, "speedup_vs_1shot": vb / v1,
            "batched_s": t_b, "single_shot_s": t_1,
            "single_shot_sample": "%d single-shot runs back to back, mean" % single_shots,
            "shot0_bitwise_equal_to_single_run": same}


def leg_orders(P, stream, fast, nsteps=2000, reps=3):
    """Work-list orders of the step kernel: rows (the default with FAST
    stencils) against balanced (the same tiles with the edge tiles spread
    evenly through the list; the EXACT default), on the benchmark shot and on
    one 1001x1001 shot.  One solver per order, each warmed once; the orders alternate over
    reps runs of nsteps steps from a reset shot.  Results must be equal bit
    for bit: only the order of independent tiles differs."""
    from poe2d_gb300 import _lib as L
    orders = {"rows": L.ORDER_ROWS, "balanced": L.ORDER_BALANCED}
    g2, coef2, px2, pz2, src2, rec2, _ = workload()
    g1, coef1, px1, pz1, srcs1, rec1 = shots_model(1)
    out = {}
    for label, (g, coef, px, pz, src, rec) in (
            ("2001x2001 benchmark shot, 40-cell C-PML", (g2, coef2, px2, pz2, src2, rec2)),
            ("one 1001x1001 shot, 30-cell C-PML", (g1, coef1, px1, pz1, srcs1[0], rec1))):
        cells = (g.NX + 1) * (g.NZ + 1)
        solvers = {}
        for name, o in orders.items():
            s = P.Solver(g, coef, px, pz, stream=stream.cuda_stream, fast=fast)
            s.add_shot(src, rec)
            s.tune(o, 64)
            s.run(64)                                # graph capture, first touch
            solvers[name] = s
        t = {name: 0.0 for name in orders}
        traces = {}
        for r in range(reps):
            for name, s in solvers.items():
                s.reset_shot(0)
                t[name] += timed(stream, lambda: s.run(nsteps))
                if r == 0:
                    traces[name] = s.traces()
        for s in solvers.values():
            s.close()
        res = {name + "_gcells": cells * nsteps * reps / t[name] / 1e9 for name in orders}
        res["balanced_vs_rows"] = t["rows"] / t["balanced"]
        res["bitwise_equal"] = bool(np.array_equal(traces["rows"].view(np.uint32),
                                                   traces["balanced"].view(np.uint32)))
        out[label] = res
    out["sample"] = "%d runs of %d steps per order, alternating, 64-step graphs" % (reps, nsteps)
    return out


def leg_uneven(P, stream, fast, nmodels, seed=7):
    """The uneven batch: nmodels independent patchy realisations, side
    U[256, 1536], steps 4 x side, one centre-surface shot each with 128
    receivers x (vx, vz, p); one batch against back-to-back single runs."""
    from poe2d_gb300 import datagen as D
    specs = D.uneven_specs(seed, 256)[:nmodels]
    t0 = time.perf_counter()
    solvers, steps = [], []
    work = 0
    for sp in specs:
        g, coef, px, pz, src, rec, ids = D.build_model(sp)
        s = P.Solver(g, coef, px, pz, stream=stream.cuda_stream, fast=fast)
        s.add_shot(src, rec)
        solvers.append(s)
        steps.append(sp["steps"])
        work += (g.NX + 1) * (g.NZ + 1) * sp["steps"]
    setup = time.perf_counter() - t0
    batch = P.Batch(solvers, stream=stream.cuda_stream)
    batch.run([64] * len(solvers))               # warm-up: graph capture, first touch
    for s in solvers:
        s.reset_shot(0)
    l0 = batch.launches
    t_b = timed(stream, lambda: batch.run(steps))
    launches = batch.launches - l0
    batch.sync()
    tr_b = [s.traces(0) for s in solvers[:4]]
    batch.close()
    for s, n in zip(solvers, steps):             # warm each context's own graph
        s.reset_shot(0)
        s.run(64)
        s.reset_shot(0)

    def singles():
        for s, n in zip(solvers, steps):
            s.run(n)
    t_1 = timed(stream, singles)
    same = all(np.array_equal(s.traces(0).view(np.uint32), t.view(np.uint32)) for s, t in zip(solvers, tr_b))
    for s in solvers:
        s.close()
    sides = [sp["side"] for sp in specs]
    return {"workload": "%d of the 256 uneven patchy models (seed %d): side U[256,1536] (here %d-%d), steps 4 x side, "
                        "20-cell C-PML, 1 shot x 128 receivers x (vx,vz,p)" % (nmodels, seed, min(sides), max(sides)),
            "cell_updates": work, "batched_gcells": work / t_b / 1e9, "back_to_back_gcells": work / t_1 / 1e9,
            "speedup_vs_back_to_back": t_1 / t_b, "batched_s": t_b, "back_to_back_s": t_1,
            "batched_launches": launches, "setup_s": setup, "first4_bitwise_equal_to_single_runs": same}


def leg_surrogate(stream, solver_gathers_per_s, members=4, batch=256, reps=5):
    """Inference throughput of the surrogate ensemble: every member's forward
    pass over a batch of 256 inputs on the tensor cores (the weights do not
    change the work; accuracy comes from poe2d_gb300.train_surrogate)."""
    import torch
    from poe2d_gb300.surrogate import CHANNELS, SAMPLES, Surrogate, forward_flops_per_sample
    nets = [Surrogate(max_batch=batch, seed=k, stream=stream.cuda_stream) for k in range(members)]
    g = torch.Generator().manual_seed(0)
    maps = torch.rand((batch, 64, 64, 2), generator=g).to(torch.bfloat16).cuda()
    sc = torch.rand((batch, 3), generator=g).cuda()
    out = torch.empty((members, batch, SAMPLES, CHANNELS), device="cuda")

    def run():
        for k, net in enumerate(nets):
            net.forward(maps, sc, out=out[k])
    run()
    run()
    t = timed(stream, lambda: [run() for _ in range(reps)]) / reps
    for net in nets:
        net.close()
    flops = forward_flops_per_sample() * batch * members
    return {"forward_gathers_per_s": batch / t, "members": members, "batch": batch, "s_per_batch": t,
            "tensor_tflops": flops / t / 1e12, "solver_gathers_per_s": solver_gathers_per_s,
            "forward_speedup_vs_solver": (batch / t) / solver_gathers_per_s if solver_gathers_per_s else None,
            "forward_sample": "inference speed of the ensemble's forward passes (the weights do not change the "
                              "work); not an accuracy-gated figure",
            "solver_sample": "the uneven batch above: models per second of the batched solver",
            "config5": config5_record()}


def config5_record():
    """Configuration 5 (20000 training, 1000 held-out models of the uneven
    family), measured by train_surrogate at its size, which takes about 40
    GPU-minutes and so runs outside the bench: the committed summary of that
    run, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "surrogate_configuration5_20000_models.json")) as f:
            r = json.load(f)
    except (OSError, ValueError):
        return None
    return {"met": bool(r["accepted_within_5pct"] > 0 and r["surrogate_speedup_vs_solver"] >= 100),
            "train_models": r["train_models"], "heldout_models": r["heldout_models"],
            "heldout_rel_l2_median": r["heldout_rel_l2_all"]["median"],
            "heldout_rel_l2_p90": r["heldout_rel_l2_all"]["p90"],
            "accepted": r["accepted"], "surrogate_speedup_vs_solver": r["surrogate_speedup_vs_solver"],
            "with_fallback_speedup_vs_solver": r["with_fallback_speedup_vs_solver"],
            "source": "python -m poe2d_gb300.train_surrogate --train 20000 --heldout 1000 --epochs 30 --batch 64 "
                      "(profiles/surrogate_configuration5_20000_models.md); narrow_family_gate below is a "
                      "narrower family, not configuration 5"}


def leg_surrogate_accuracy(stream):
    """Accuracy of the whole learned pipeline on the family it learns: 256 x
    256 water-saturated grids of porosity 0.2, f0 drawn from [150, 300] Hz;
    128 training and 32 held-out gathers from the batched solver, 4 members
    trained on the tensor cores, held-out models answered by the ensemble mean
    where the members agree within 5 % and by the solver elsewhere."""
    import contextlib
    import io
    import torch
    from poe2d_gb300 import train_surrogate as T
    keep = torch.cuda.current_stream()
    try:
        with contextlib.redirect_stdout(io.StringIO()):          # the trainer prints its own summary line
            s = T.main(["--train", "128", "--heldout", "32", "--epochs", "1500", "--gas-max", "0", "--side-min",
                        "256", "--side-max", "256", "--phi", "0.2", "0.2", "--f0", "150", "300"])
    finally:
        torch.cuda.set_stream(keep)
    return {"family": "256x256 water-saturated grids, porosity 0.2, f0 U[150, 300] Hz (no gas patches)",
            "train_models": s["train_models"], "heldout_models": s["heldout_models"], "members": s["members"],
            "threshold": s["threshold"], "accepted": s["accepted"], "accepted_rel_l2": s["accepted_rel_l2"],
            "heldout_rel_l2_all": s["heldout_rel_l2_all"],
            "surrogate_speedup_vs_solver": s["surrogate_speedup_vs_solver"],
            "with_fallback_speedup_vs_solver": s["with_fallback_speedup_vs_solver"], "wall_s": s["wall_s"]}


def alg_bytes_per_step(g, s_ctx_strips, per_cell=96):
    """Algorithmic HBM bytes of one time step: per_cell bytes per cell plus
    8 B per C-PML memory variable on its strip (6 on x strips, 6 on z strips).
    per_cell = 96: 8 FP32 state fields read+written + 8 coefficient planes read.
    per_cell = 73: what the palette kernel must move at least -- the 9
    integrated state fields (vx vz wx wz sigma_xz g11 g22 xi1 xi2) read and
    written (72 B) and a 1-byte material id."""
    nx, nz = g.NX + 1, g.NZ + 1
    wx, hz = s_ctx_strips
    return per_cell * nx * nz + 48 * nz * wx + 48 * nx * hz


def strip_extent(px, pz):
    def ext(prof):
        n1 = prof.shape[1]
        a = (prof[0] != 0) | (prof[3] != 0)
        lo = max([i + 1 for i in range(n1 // 2) if a[i]], default=0)
        hi = min([i for i in range(n1 // 2, n1) if a[i]], default=n1)
        return n1 if lo >= hi else lo + (n1 - hi)
    return ext(px), ext(pz)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                smax = float(p[1])
            except ValueError:
                continue
            for n, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


class CpuOracle:
    """The oracle on the host cores over the bench model (bounded step samples)."""

    def __init__(self, g, coef, px, pz, src_ix, src_iz, threads=None):
        from oracle import oracle as O
        O.build()
        self.th = threads or os.cpu_count() or 1
        self.o = O.Oracle(O.REFMIXED, g.NX, g.NZ, g.dx, g.dz, g.dt, coef, px, pz, threads=self.th)
        tab = O.source_table(1, F0, g.dt, NSTEPS, amplitude=1e6, t_cut=0.0, dx=g.dx, dz=g.dz)
        self.o.set_source(src_ix, src_iz, O.SRC_FZ, tab)
        self.o.set_receivers([(src_ix, src_iz, 1)])
        self.cells = (g.NX + 1) * (g.NZ + 1)
        self.o.run(2)                     # first touch of every page, thread start-up
        t0 = time.perf_counter()
        self.o.run(2)
        self.per_step = (time.perf_counter() - t0) / 2

    def sample(self, seconds):
        n = int(min(max(2, seconds / max(self.per_step, 1e-6)), 5000))
        t0 = time.perf_counter()
        self.o.run(n)
        el = time.perf_counter() - t0
        return n, el


def cpu_sample(g, coef, px, pz, src_ix, src_iz, target_s=12.0):
    c = CpuOracle(g, coef, px, pz, src_ix, src_iz)
    n, el = c.sample(target_s)
    return {"value": c.cells * n / el / 1e9, "unit": "Gcell-updates/s", "cores": c.th, "kind": "port",
            "sample": "%d of the %d steps of the 2001x2001 shot (after 4 untimed), %.1f s" % (n, NSTEPS, el)}


def padded_ids(n=2010, seed=0):
    """The benchmark model's patchy ids on the n x n grid the reference's own
    programs need (a multiple of 10 cells per side, cu:1597-1600)."""
    from poe2d_gb300.patchy import random_patches
    return random_patches((n, n), DX, fraction=0.10, r_min=2.0, r_max=10.0, seed=1234 + seed)


def reference_gpu_leg():
    """The reference's own CUDA program (staged by baseline/stage_ref.sh) on
    this GPU, 2000 steps of the benchmark model padded to 2010 x 2010."""
    from baseline import ref_programs as R
    if not R.staged():
        return {"unavailable": "the reference's sources are not staged (baseline/stage_ref.sh needs the reference tree)"}
    try:
        return R.time_cuda(padded_ids(), DX, DT, NPML, F0, nstep=2000, samp=1000)
    except Exception as exc:                       # reported, never fatal to the bench line
        return {"unavailable": repr(exc)[:300]}


def reference_cpu_program_leg():
    """The reference's own serial C++ program on one host core, one chunk of
    51 steps of the benchmark model padded to 2010 x 2010."""
    from baseline import ref_programs as R
    if not R.staged():
        return {"unavailable": "the reference's sources are not staged (baseline/stage_ref.sh needs the reference tree)"}
    try:
        return R.time_cpu(padded_ids(), DX, DT, NPML, F0, samp=50)
    except Exception as exc:
        return {"unavailable": repr(exc)[:300]}


def bench_config(ids, ws):
    """The workload both arms report (the same dict for ours and the reference)."""
    return {"workload": "2001x2001 patchy gas/water sandstone shot, h=0.5 m, 40-cell C-PML, dt=5e-5 s, "
                        "20000 steps, Ricker 200 Hz vertical force, 400 receivers x (vx,vz,p)",
            "grid": [NX + 1, NZ + 1], "time_steps": NSTEPS, "pml": NPML, "receivers": NREC,
            "gas_fraction": float(ids.mean()), "parallelism": "replicas" if ws > 1 else "single",
            "l2": "inputs larger than L2 (12 state planes x 16 MB + 8 coefficient planes)"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args, ws, rank):
    """CPU reference arm: the oracle's restatement of the reference loop
    (REFMIXED: bit for bit the reference's own kernel lines where those build
    on the host), OpenMP over all host threads, on the benchmark shot.  Its
    inputs come from the oracle's own set-up restatements, not the library.
    Each bench step is a ~5 s sample of the shot's time steps; ms_per_step is
    the measured time of one such step."""
    if rank != 0:
        return
    g, coef, px, pz, src, rec, ids = workload(via="oracle")
    c = CpuOracle(g, coef, px, pz, src.ix, src.iz)
    for _ in range(args.warmup):
        c.o.run(1)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        n, el = c.sample(5.0)
        tot_n += n
        tot_t += el
    value = c.cells * tot_n / tot_t / 1e9
    sample = ("%d bench steps, each a ~5 s sample (~%d of the %d time steps of the 2001x2001 shot), %.1f s total; "
              "the full shot would take %.0f s" % (args.steps, tot_n // max(args.steps, 1), NSTEPS, tot_t,
                                                     c.cells * NSTEPS / (value * 1e9)))
    ref_prog = reference_cpu_program_leg() if not args.no_ref_programs else None
    line = {"metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot_t / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": bench_config(ids, ws),
            "arm": "CPU oracle (C restatement of the reference loop, bit-exact with the reference's own code where "
                   "that builds), OpenMP over all host threads",
            "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": c.th, "kind": "port",
                             "sample": sample},
            "reference_cpu_program": ref_prog,
            "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    global NPML
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--stencil", default="fast", choices=["fast", "exact"],
                    help="fast: plain FP32 stencils; exact: FP32 arithmetic rounded like the reference's FP64 lines")
    ap.add_argument("--no-parity", action="store_true", help="skip the fast-vs-exact drift check")
    ap.add_argument("--no-orders", action="store_true", help="skip the work-list order comparison")
    ap.add_argument("--pml", type=int, default=40,
                    help="C-PML width in cells of the single-shot workload (profiling; the benchmark is 40)")
    ap.add_argument("--no-ref-programs", action="store_true",
                    help="skip timing the reference's own CUDA (ours) and serial C++ (reference arm) programs")
    ap.add_argument("--no-surrogate-train", action="store_true",
                    help="skip training and scoring the surrogate ensemble on its narrow family")
    ap.add_argument("--batched", type=int, default=64, metavar="M",
                    help="batched legs: 64 shots of one 1001x1001 model, and M of the 256 uneven models "
                         "(0 skips both)")
    args = ap.parse_args()
    NPML = args.pml
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    import poe2d_gb300 as P
    from poe2d_gb300 import build as B
    B.build()

    g, coef, px, pz, src, rec, ids = workload(seed=0, shift=8 * rank)
    # a real (non-default) stream: the solver's kernels and the timing events
    # must be on the same stream (handle 0 would give the solver a private one)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    fast = args.stencil == "fast"
    solver = P.Solver(g, coef, px, pz, stream=stream.cuda_stream, fast=fast)
    solver.add_shot(src, rec)
    cells = (g.NX + 1) * (g.NZ + 1)

    def shot():
        solver.reset_shot(0)
        solver.run(NSTEPS)

    for _ in range(args.warmup):
        shot()
    torch.cuda.synchronize()
    launches0 = solver.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        ev0.record(stream)
        for _ in range(args.steps):
            shot()
        ev1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if pg:
        pg.barrier()
    ms = ev0.elapsed_time(ev1)
    launches = solver.launches - launches0
    t = torch.tensor([ms], device="cuda")
    if pg:
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
    ms_max = float(t.item())
    total_cells = cells * NSTEPS * args.steps * ws
    value = total_cells / (ms_max * 1e-3) / 1e9

    # roofline of the time step: algorithmic bytes per step / time per step
    hbm, peak_kind = peaks()
    alg = alg_bytes_per_step(g, strip_extent(px, pz))
    alg_pal = alg_bytes_per_step(g, strip_extent(px, pz), per_cell=73)
    step_s = ms * 1e-3 / (args.steps * NSTEPS)
    achieved = alg / step_s / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "k_tile_pal_traffic_2001x2001.json")) as f:
            tr = json.load(f)
        traffic = float(tr["dram_bytes_per_cell_update"]) * cells
    except Exception:
        pass
    trace = solver.traces()
    ok = bool(np.isfinite(trace).all() and np.abs(trace).max() > 0)
    tuning = solver.tuning()            # the library's defaults for this shot

    # drift of this run's traces against the other stencil rounding, same shot
    parity = None
    if not args.no_parity:
        other = P.Solver(g, coef, px, pz, stream=stream.cuda_stream, fast=not fast)
        other.add_shot(src, rec)
        other.run(NSTEPS)
        tr2 = other.traces()
        other.close()
        comp = {}
        for ci, name in enumerate(("vx", "vz", "p")):
            a = trace[:, ci * NREC:(ci + 1) * NREC].astype(np.float64)
            b = tr2[:, ci * NREC:(ci + 1) * NREC].astype(np.float64)
            comp[name] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
        parity = {"rel_l2_vs_" + ("exact" if fast else "fast") + "_stencils": comp, "tolerance": 1e-5,
                  "steps": NSTEPS}

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hcoef = torch.empty(coef.shape, dtype=torch.float32, pin_memory=True).numpy()
        hcoef[...] = coef
        htr = torch.empty((NSTEPS, len(rec)), dtype=torch.float32, pin_memory=True).numpy()
        solver.close()
        e2e_steps = max(1, args.steps)
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            s2 = P.Solver(g, hcoef, px, pz, stream=stream.cuda_stream, fast=fast)
            s2.add_shot(src, rec)
            s2.run(NSTEPS)
            P._lib.check(P.lib().poe_get_traces(s2.h, 0, htr.ctypes.data_as(P.solver._fp), htr.size), s2.h)
            s2.close()
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        te = torch.tensor([el], device="cuda")
        if pg:
            pg.all_reduce(te, op=pg.ReduceOp.MAX)
        el = float(te.item())
        e2e = {"value": cells * NSTEPS * e2e_steps * ws / el / 1e9, "unit": "Gcell-updates/s",
               # what the calls upload: material ids (1 B per cell, the palette
               # is built on the host from the coefficient planes), the C-PML
               # profiles, the receiver list and the source table
               "h2d_bytes_per_step": int(ids.size + px.nbytes + pz.nbytes + 16 * len(rec) + 4 * NSTEPS),
               "d2h_bytes_per_step": int(htr.nbytes)}
    else:
        solver.close()

    batched = None
    surrogate = None
    if args.batched > 0:
        batched = {"shots": leg_shots(P, stream, fast), "uneven": leg_uneven(P, stream, fast, args.batched)}
        un = batched["uneven"]
        surrogate = leg_surrogate(stream, args.batched / un["batched_s"])
        if not args.no_surrogate_train:
            surrogate["narrow_family_gate"] = leg_surrogate_accuracy(stream)

    orders = None
    if rank == 0 and not args.no_orders:
        try:
            orders = leg_orders(P, stream, fast)
        except Exception as exc:                     # reported, never fatal to the bench line
            orders = {"error": repr(exc)[:300]}

    cb = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_sample(g, coef, px, pz, src.ix, src.iz)
    ref_gpu = None
    if rank == 0 and ws == 1 and not args.no_ref_programs:
        ref_gpu = reference_gpu_leg()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(ids, ws),
            "stencil_rounding": ("plain FP32 stencils" if fast else
                                 "exact: FP64 sub-expressions of the reference rounded once"),
            "coefficients": "material palette (1-byte id per cell, 2 materials)",
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_step": alg, "step_us": step_s * 1e6,
                         "palette_min_bytes_per_step": alg_pal,
                         "palette_frac": alg_pal / step_s / 1e9 / hbm,
                         "per": "time step: one step-spanning launch of the step kernel runs 64 steps; "
                                "traffic = ncu's DRAM bytes of a warm launch / 64"},
            "cpu_baseline": cb, "reference_gpu": ref_gpu, "e2e": e2e, "gpu_launches": launches,
            "tuning": tuning,
            "clocks": clk.summary(), "wall_s": wall, "finite": ok, "parity": parity, "batched": batched,
            "surrogate": surrogate, "orders": orders,
        }
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()

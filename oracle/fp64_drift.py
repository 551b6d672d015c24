"""FP32 drift of the benchmark workloads against an FP64 run of the
reference loop.

For each workload the GPU runs the shot with EXACT stencils (the reference's
FP32 storage with FP64 stencil temporaries, bit for bit) and with FAST
stencils (plain FP32), and the oracle runs the same inputs in F64 on the host
cores.  One JSON line per shot gives the relative L2 error of the traces
against F64 and the largest trace error relative to the trace peak.

    python oracle/fp64_drift.py                                     # all four
    python oracle/fp64_drift.py --workloads sandstone201,shots1001  # a subset

Workloads (synthetic, seeded):
  sandstone201  201 x 201 homogeneous water-saturated sandstone, 20-cell
                C-PML, 2000 steps, vertical-force Ricker at the centre, 11
                receivers 40 cells above
  patchy2001    the 2001 x 2001 patchy benchmark shot, 40-cell C-PML, 20000
                steps, 400 surface receivers
  shots1001     shot 0 of the 64-shot batch: 1001 x 1001 patchy model,
                30-cell C-PML, 10000 steps, 256 surface receivers
  uneven4       the first four models of the uneven batch (seed 7): side
                U[256, 1536], steps 4 x side, 128 surface receivers each

Test infrastructure: it runs the oracle (needs a CUDA device and the built
oracle library).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def sandstone_201():
    import poe2d_gb300 as P
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = P.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    n = 200
    ids = np.zeros((n + 1, n + 1), np.uint8)
    coef, vp = P.coeffs_biot([water], ids)
    g = P.grid(n, n, 0.5, 5e-5)
    P.check_courant(g, vp)
    px, pz = P.pml_profiles(g, 20, 200.0, vp)
    src = P.source(100, 100, P.SRC_RICKER_FZ, 200.0, 1e6, 0.0)
    rec = [(x, 60, c) for c in (P.REC_VX, P.REC_VZ, P.REC_P) for x in range(50, 151, 10)]
    return [("201^2 sandstone, 2000 steps", g, coef, px, pz, src, rec, 2000)]


def benchmark_2001():
    import bench
    g, coef, px, pz, src, rec, _ = bench.workload()
    return [("2001^2 patchy shot, 20000 steps", g, coef, px, pz, src, rec, bench.NSTEPS)]


def shots_1001():
    import bench
    g, coef, px, pz, srcs, rec = bench.shots_model(64, 1001, 30, 256)
    return [("1001^2 patchy model, shot 0 of 64, 10000 steps", g, coef, px, pz, srcs[0], rec, 10000)]


def uneven_4():
    from poe2d_gb300 import datagen as D
    out = []
    for sp in D.uneven_specs(7, 256)[:4]:
        g, coef, px, pz, src, rec, _ = D.build_model(sp)
        out.append(("uneven model %d, side %d, %d steps" % (sp["index"], sp["side"], sp["steps"]),
                    g, coef, px, pz, src, rec, sp["steps"]))
    return out


WORKLOADS = {"sandstone201": sandstone_201, "patchy2001": benchmark_2001, "shots1001": shots_1001,
             "uneven4": uneven_4}


def gpu_traces(g, coef, px, pz, src, rec, nsteps, fast):
    import poe2d_gb300 as P
    with P.Solver(g, coef, px, pz, fast=fast) as s:
        s.add_shot(src, rec)
        s.run(nsteps)
        return s.traces().astype(np.float64)


def f64_traces(g, coef, px, pz, src, rec, nsteps):
    from oracle import oracle as O
    o = O.Oracle(O.F64, g.NX, g.NZ, g.dx, g.dz, g.dt, coef, px, pz)
    where = O.SRC_FZ if src.kind == 1 else O.SRC_P
    o.set_source(src.ix, src.iz, where, O.source_table(src.kind, src.f0, g.dt, nsteps, amplitude=src.amplitude,
                                                       t_cut=src.t_cut, dx=g.dx, dz=g.dz))
    o.set_receivers(np.asarray(rec, np.int32))
    return o.run(nsteps).astype(np.float64)


def drift(t, ref):
    return {"rel_l2": float(np.linalg.norm(t - ref) / np.linalg.norm(ref)),
            "max_err_over_peak": float(np.abs(t - ref).max() / np.abs(ref).max())}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workloads", default=",".join(WORKLOADS))
    args = ap.parse_args(argv)
    from oracle import oracle as O
    O.build()
    for w in args.workloads.split(","):
        for name, g, coef, px, pz, src, rec, nsteps in WORKLOADS[w]():
            t0 = time.perf_counter()
            ref = f64_traces(g, coef, px, pz, src, rec, nsteps)
            t_cpu = time.perf_counter() - t0
            ex = gpu_traces(g, coef, px, pz, src, rec, nsteps, False)
            fa = gpu_traces(g, coef, px, pz, src, rec, nsteps, True)
            print(json.dumps({"workload": name, "cells": (g.NX + 1) * (g.NZ + 1), "steps": nsteps,
                              "receivers": len(rec), "exact_vs_f64": drift(ex, ref), "fast_vs_f64": drift(fa, ref),
                              "fast_vs_exact": drift(fa, ex), "f64_cpu_s": round(t_cpu, 1),
                              "f64_threads": os.cpu_count()}), flush=True)


if __name__ == "__main__":
    main()

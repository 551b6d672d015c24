"""Seeded synthetic workloads: patchy models of uneven sizes for batched runs
and surrogate training data.

The reference (thejatmik/poe2d) generates its models with patchymodel.m
(deterministic circle lattices, patchy:17-260) and runs one model per
process.  The batched workloads here are random realisations of the same
kind of medium: a sandstone frame saturated with water, with circular gas
patches.  Every draw comes from numpy's PCG64 seeded per model, so a
(seed, index) pair always gives the same model.

``uneven_specs(seed, n)``  per-model parameters: grid side U[256, 1536],
    steps 4 x side, porosity U[0.1, 0.3], gas fraction U[0, 0.3], mean patch
    radius U[1, 10] m, f0 U[150, 300] Hz.
``patchy_ids(...)``        vectorised circle rasteriser (gas = 1).
``build_model(spec)``      grid, coefficients, profiles, source, receivers.
``resample(traces, m)``    traces (steps x channels) linearly resampled to m samples.
"""
from __future__ import annotations

import numpy as np

FRAME = dict(rho_s=2650.0, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
WATER = dict(rho_f=1000.0, k_f=2.25e9, eta=1e-3)
GAS = dict(rho_f=100.0, k_f=0.02e9, eta=1e-5)
DX, DT = 0.5, 5e-5


def patchy_ids(shape, dx, fraction, r_mean, seed, spread=0.5):
    """uint8 ids (0 background, 1 gas) with random circles of radius
    U[(1-spread) r_mean, (1+spread) r_mean] metres until the gas area reaches
    ``fraction`` of the grid.  Circles are drawn in rounds sized from the
    area still missing, and rasterised for a whole round at once."""
    nz, nx = shape
    ids = np.zeros(shape, np.uint8)
    if fraction <= 0:
        return ids
    rng = np.random.default_rng(seed)
    target = fraction * nz * nx
    r_lo, r_hi = (1 - spread) * r_mean / dx, (1 + spread) * r_mean / dx
    mean_area = np.pi * (r_lo * r_lo + r_lo * r_hi + r_hi * r_hi) / 3.0
    have = 0
    for _ in range(200):
        missing = target - have
        if missing <= 0:
            break
        m = int(max(4, min(200000, 0.6 * missing / max(mean_area, 1.0))))
        rc = rng.uniform(r_lo, r_hi, m)
        cz = rng.uniform(0, nz, m)
        cx = rng.uniform(0, nx, m)
        R = int(np.ceil(rc.max()))
        iz0, ix0 = np.floor(cz).astype(np.int64), np.floor(cx).astype(np.int64)
        for dz in range(-R, R + 2):
            z = iz0 + dz
            okz = (z >= 0) & (z < nz)
            ddz = (z - cz) ** 2
            for dxx in range(-R, R + 2):
                x = ix0 + dxx
                hit = okz & (x >= 0) & (x < nx) & (ddz + (x - cx) ** 2 <= rc * rc)
                if hit.any():
                    ids[z[hit], x[hit]] = 1
        have = int(np.count_nonzero(ids))
    return ids


def uneven_specs(seed, n, n_min=256, n_max=1536, gas_max=0.3, phi=(0.1, 0.3), f0=(150.0, 300.0)):
    """n model specifications of the uneven batch (one row per model).
    The ranges narrow the family (e.g. gas_max = 0: homogeneous
    water-saturated models)."""
    rng = np.random.default_rng(seed)
    side = rng.integers(n_min, n_max + 1, n)
    out = []
    for i in range(n):
        out.append(dict(index=i, seed=int(seed) * 100003 + i, side=int(side[i]), steps=4 * int(side[i]),
                        phi=float(rng.uniform(phi[0], phi[1])), gas=float(rng.uniform(0.0, gas_max)),
                        radius=float(rng.uniform(1.0, 10.0)), f0=float(rng.uniform(f0[0], f0[1]))))
    return out


def materials(phi):
    import poe2d_gb300 as P
    water = P.biot_material(phi=phi, **FRAME, **WATER)
    gas = P.biot_material(phi=phi, **FRAME, **GAS)
    return [water, gas]


def build_model(spec, npml=20, nrec=128, comps=(0, 1, 2)):
    """Everything a Solver needs for one model of the uneven batch:
    (grid, coef, prof_x, prof_z, source, receivers, ids).  A vertical-force
    Ricker at the surface centre (row npml) and nrec receivers along the same
    row between the C-PML strips, each recording the components ``comps``
    (0 vx, 1 vz, 2 p; receiver-major within a component)."""
    import poe2d_gb300 as P
    n = spec["side"]
    NX = NZ = n - 1
    ids = patchy_ids((n, n), DX, spec["gas"], spec["radius"], spec["seed"])
    coef, vp = P.coeffs_biot(materials(spec["phi"]), ids)
    g = P.grid(NX, NZ, DX, DT)
    P.check_courant(g, vp)
    px, pz = P.pml_profiles(g, npml, spec["f0"], vp)
    src = P.source(n // 2, npml, P.SRC_RICKER_FZ, spec["f0"], 1e6, 0.0)
    xs = npml + 1 + (np.arange(nrec) * (NX - 2 * npml - 2)) // (nrec - 1)
    rec = [(int(x), npml, c) for c in comps for x in xs]
    return g, coef, px, pz, src, rec, ids


def resample(traces, m):
    """(steps, channels) -> (m, channels), linear interpolation on a uniform
    time axis spanning the same duration (first and last samples kept)."""
    t = np.asarray(traces, np.float32)
    n = t.shape[0]
    if n == m:
        return t.copy()
    pos = np.linspace(0.0, n - 1, m)
    i0 = np.minimum(np.floor(pos).astype(np.int64), n - 2)
    w = (pos - i0).astype(np.float32)[:, None]
    return (1.0 - w) * t[i0] + w * t[i0 + 1]

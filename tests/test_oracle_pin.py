"""Pin the CPU oracle: bit-for-bit against the reference's own code.

The golden fixtures were produced by tests/golden/make_golden.py from the
reference's kernels and set-up lines compiled for the host; where that
harness is built (a tree with the reference sources) the oracle is also
compared with it directly on further cases.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def ref_rec_list(NX, NZ, isrc, jsrc, panj, panj2, a0, a1):
    L2, L = (NZ + 1) // panj, (NX + 1) // panj2
    rec = [(isrc, k * L2 - 1, 1) for k in range(1, panj + 1)]
    rec += [(isrc, k * L2 - 1, 0) for k in range(1, panj + 1)]
    rec += [(k * L - 1, 10, 1) for k in range(1, panj2 + 1)]
    rec += [(k * L - 1, 10, 0) for k in range(1, panj2 + 1)]
    xc = (NX + 1) // 2 - 1
    rec += [(xc, y, 1) for y in (50, a0, a1, jsrc)]
    return rec


def ref_seis_concat(d):
    return np.concatenate([d["seismo"], d["deismo"], d["seismo1"], d["deismo1"], d["seismo0"], d["seismo2"],
                           d["seismo3"], d["seismo4"]], axis=1)


def test_oracle_setup_matches_golden(oracle_mod):
    O = oracle_mod
    d = np.load(os.path.join(GOLD, "ref_setup.npz"))
    from poe2d_gb300.solver import REFERENCE_FLUID_TABLE
    coef, bad = O.coeffs_from_medium(d["medium"], d["cp"], d["cs"], d["rho"], REFERENCE_FLUID_TABLE)
    assert bad == 0
    assert bits_equal(coef, d["coef"])
    px, pz = O.pml_profiles(int(d["NX"]), int(d["NZ"]), float(d["dx"]), float(d["dx"]), float(d["dt"]),
                            int(d["npml"]), float(d["cp"].max()), f0=float(d["f0"]))
    assert bits_equal(px, d["prof_x"]) and bits_equal(pz, d["prof_z"])


def test_oracle_loop_matches_golden(oracle_mod):
    O = oracle_mod
    d = np.load(os.path.join(GOLD, "ref_loop.npz"))
    NX, NZ, n = int(d["NX"]), int(d["NZ"]), int(d["nsteps"])
    dx, dt, f0 = float(d["dx"]), float(d["dt"]), float(d["f0"])
    o = O.Oracle(O.REFMIXED, NX, NZ, dx, dx, dt, d["coef"], d["prof_x"], d["prof_z"])
    o.set_source(int(d["isrc"]), int(d["jsrc"]), O.SRC_P, O.source_table(0, f0, dt, n, t_cut=0.4))
    rec = ref_rec_list(NX, NZ, int(d["isrc"]), int(d["jsrc"]), int(d["panj"]), int(d["panj2"]), int(d["a0"]),
                       int(d["a1"]))
    # slots outside the grid (y = 50 here) stay zero in the reference
    valid = [i for i, r in enumerate(rec) if r[1] <= NZ]
    o.set_receivers([rec[i] for i in valid])
    tr = o.run(n)
    ref = ref_seis_concat(d)
    assert bits_equal(tr, ref[:, valid])
    assert not np.any(ref[:, [i for i in range(len(rec)) if i not in valid]])
    for name in O.FIELDS[:12]:
        assert bits_equal(o.field(name), d[name]), name
    assert np.abs(d["vz"]).max() > 0


@pytest.mark.parametrize("case", [
    # NX, NZ, dx, dt, npml, isrc, jsrc, nsteps
    (58, 61, 0.5, 5e-5, 6, 29, 30, 120),
    (47, 39, 1.25, 95e-6, 5, 23, 1, 90),     # source row outside stress1's rows: sigma2 accumulates
    (53, 44, 0.3, 3e-5, 6, 26, 20, 100),     # 24 h = 7.2 needs many bits: no exact float divisor
])
def test_oracle_vs_reference_harness(oracle_mod, case):
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference harness not built here")
    NX, NZ, dx, dt, npml, isrc, jsrc, n = case
    rng = np.random.default_rng(NX * 100 + NZ)
    sh = (NZ + 1, NX + 1)
    medium = rng.integers(0, 4, size=sh).astype(np.float32)
    cp = rng.uniform(2600, 3300, size=sh).astype(np.float32)
    cs = rng.uniform(1300, 1700, size=sh).astype(np.float32)
    rho = rng.uniform(2100, 2500, size=sh).astype(np.float32)
    from tests.golden.make_golden import LOOP_TABLE
    coef, _ = O.coeffs_from_medium(medium, cp, cs, rho, LOOP_TABLE)
    f0 = 150.0
    px, pz = O.pml_profiles(NX, NZ, dx, dx, dt, npml, float(cp.max()), f0=f0)
    rpx, rpz, _ = O.ref_pml(NX, NZ, dx, dx, dt, npml, f0, float(cp.max()))
    assert bits_equal(px, rpx) and bits_equal(pz, rpz)
    panj, panj2, a0, a1 = 3, 4, 9, 14
    fields, seis, ig = O.ref_run(NX, NZ, dx, dt, isrc, jsrc, f0, coef, px, pz, n, panj, panj2, a0, a1)
    assert ig == n
    o = O.Oracle(O.REFMIXED, NX, NZ, dx, dx, dt, coef, px, pz)
    o.set_source(isrc, jsrc, O.SRC_P, O.source_table(0, f0, dt, n, t_cut=0.4))
    rec = ref_rec_list(NX, NZ, isrc, jsrc, panj, panj2, a0, a1)
    valid = [i for i, r in enumerate(rec) if r[1] <= NZ]
    o.set_receivers([rec[i] for i in valid])
    tr = o.run(n)
    assert bits_equal(tr, ref_seis_concat(seis)[:, valid])
    for name in O.FIELDS:
        assert bits_equal(o.field(name), fields[name]), name


def test_fp32_drift_against_fp64_is_small(oracle_mod):
    """The FP64 yardstick: FP32 storage drifts ~1e-6 on a short run."""
    O = oracle_mod
    d = np.load(os.path.join(GOLD, "ref_loop.npz"))
    NX, NZ, n = int(d["NX"]), int(d["NZ"]), int(d["nsteps"])
    dx, dt, f0 = float(d["dx"]), float(d["dt"]), float(d["f0"])
    out = {}
    for mode in (O.REFMIXED, O.F32, O.F64):
        o = O.Oracle(mode, NX, NZ, dx, dx, dt, d["coef"], d["prof_x"], d["prof_z"])
        o.set_source(int(d["isrc"]), int(d["jsrc"]), O.SRC_P, O.source_table(0, f0, dt, n, t_cut=0.4))
        o.set_receivers([(x, z, 1) for x in range(10, 31, 5) for z in (12, 20)])
        out[mode] = o.run(n).astype(np.float64)
    ref = out[O.F64]
    for mode in (O.REFMIXED, O.F32):
        rel = np.linalg.norm(out[mode] - ref) / np.linalg.norm(ref)
        assert rel < 1e-5, (mode, rel)

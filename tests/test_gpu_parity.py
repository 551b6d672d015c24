"""GPU parity: the sm_103a kernels through the C ABI against the oracle and
the golden fixtures of the reference's own code.

Bar: the default (exact-rounding) kernels reproduce the reference's
FP32/FP64 arithmetic: against the golden run of the reference's own code
every trace value and every field is bit-identical; against the oracle on
other models, relative L2 <= 1e-6 and max |diff| <= 1e-6 x peak.  The
fast-stencil variant must meet the stated tolerance: relative L2 <= 1e-5 on
the traces and a largest snapshot error <= 1e-5 of the field's peak.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL_EXACT = 1e-6
TOL_FAST = 1e-5


def rel_l2(a, b):
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def max_rel_peak(a, b, peak):
    return float(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)).max() / peak)


def test_golden_reference_loop_on_gpu(poe):
    d = np.load(os.path.join(GOLD, "ref_loop.npz"))
    NX, NZ, n = int(d["NX"]), int(d["NZ"]), int(d["nsteps"])
    g = poe.grid(NX, NZ, float(d["dx"]), float(d["dt"]))
    rec = poe.ref_receivers(g, int(d["isrc"]), int(d["jsrc"]), int(d["panj"]), int(d["panj2"]), int(d["a0"]),
                            int(d["a1"]))
    with poe.Solver(g, d["coef"], d["prof_x"], d["prof_z"]) as s:
        s.add_shot(poe.source(int(d["isrc"]), int(d["jsrc"]), poe.SRC_REF_DGAUSS_P, float(d["f0"])), rec)
        s.run(n)
        tr = s.traces()
        ref = np.concatenate([d["seismo"], d["deismo"], d["seismo1"], d["deismo1"], d["seismo0"], d["seismo2"],
                              d["seismo3"], d["seismo4"]], axis=1)
        assert tr.shape == ref.shape
        assert np.array_equal(tr.view(np.uint32), ref.view(np.uint32)), rel_l2(tr, ref)
        for name in ("vx", "vz", "wx", "wz", "sxx", "szz", "sxz", "p", "g11", "g22", "xi1", "xi2"):
            f = s.field(name)
            assert np.array_equal(f.view(np.uint32), d[name].view(np.uint32)), (name, max_rel_peak(
                f, d[name], max(np.abs(d[name]).max(), 1e-30)))
        assert s.launches > 0


def _case(poe, O, NX, NZ, dx, dt, npml, f0, seed, table):
    rng = np.random.default_rng(seed)
    sh = (NZ + 1, NX + 1)
    medium = rng.integers(0, 4, size=sh).astype(np.float32)
    cp = rng.uniform(2600, 3300, size=sh).astype(np.float32)
    cs = rng.uniform(1300, 1700, size=sh).astype(np.float32)
    rho = rng.uniform(2100, 2500, size=sh).astype(np.float32)
    g = poe.grid(NX, NZ, dx, dt)
    coef = poe.coeffs_from_medium(g, medium, cp, cs, rho, table)
    px, pz = poe.pml_profiles(g, npml, f0, float(cp.max()))
    return g, coef, px, pz


@pytest.mark.parametrize("fast", [False, True])
def test_two_shots_vs_oracle(poe, oracle_mod, fast):
    """Two shots in one context (pressure dGauss and vertical-force Ricker),
    recording vx, vz and p; 150 steps = two graph replays + a direct tail."""
    O = oracle_mod
    from tests.golden.make_golden import LOOP_TABLE
    NX, NZ, dx, dt, npml, f0, n = 95, 77, 0.5, 5e-5, 12, 200.0, 150
    g, coef, px, pz = _case(poe, O, NX, NZ, dx, dt, npml, f0, 3, LOOP_TABLE)
    rec = [(x, 30, c) for c in (0, 1, 2) for x in range(14, 82, 9)]
    shots = [(poe.source(40, 38, poe.SRC_REF_DGAUSS_P, f0, 1.0, 0.4), O.SRC_P, 0, 0.4, 1.0),
             (poe.source(55, 20, poe.SRC_RICKER_FZ, f0, 1e3, 0.0), O.SRC_FZ, 1, 0.0, 1e3)]
    with poe.Solver(g, coef, px, pz, fast=fast) as s:
        for src, *_ in shots:
            s.add_shot(src, rec)
        s.run(100)
        s.run(50)
        for i, (src, where, kind, tcut, amp) in enumerate(shots):
            o = O.Oracle(O.F32 if fast else O.REFMIXED, NX, NZ, dx, dx, dt, coef, px, pz)
            o.set_source(src.ix, src.iz, where, O.source_table(kind, f0, dt, n, amplitude=amp, t_cut=tcut, dx=dx,
                                                               dz=dx))
            o.set_receivers(rec)
            ref = o.run(n)
            tr = s.traces(i)
            tol = TOL_FAST if fast else TOL_EXACT
            for c in range(3):
                sl = slice(c * 8, (c + 1) * 8)
                assert rel_l2(tr[:, sl], ref[:, sl]) <= tol, (i, c, rel_l2(tr[:, sl], ref[:, sl]))
            for name in ("vz", "p", "sxz", "wx"):
                r = o.field(name)
                err = max_rel_peak(s.field(name, i), r, np.abs(r).max())
                assert err <= tol, (i, name, err)


def test_reset_reproduces_and_fields_roundtrip(poe, oracle_mod):
    from tests.golden.make_golden import LOOP_TABLE
    NX, NZ = 60, 50
    g, coef, px, pz = _case(poe, oracle_mod, NX, NZ, 0.5, 5e-5, 8, 200.0, 11, LOOP_TABLE)
    rec = [(30, 20, 1), (31, 21, 2)]
    with poe.Solver(g, coef, px, pz) as s:
        s.add_shot(poe.source(30, 25, poe.SRC_RICKER_FZ, 200.0, 1.0, 0.0), rec)
        s.run(70)
        a = s.traces().copy()
        s.reset_shot(0)
        assert s.steps() == 0 and not np.any(s.field("vz"))
        s.run(70)
        assert np.array_equal(a, s.traces())
        v = np.random.default_rng(0).standard_normal((NZ + 1, NX + 1)).astype(np.float32)
        s.set_field("wz", v)
        assert np.array_equal(s.field("wz"), v)
        st, mx = s.check_finite(0)
        assert st == 0 and mx > 0
        with pytest.raises(poe.PoeError):
            s.set_field("p", v)          # derived from g11 g22 xi1 xi2, not settable
        s.set_field("sxz", np.full((NZ + 1, NX + 1), np.nan, np.float32))
        st, _ = s.check_finite(0)
        assert st == 3


def _patchy(poe, NX, NZ, seed):
    from poe2d_gb300.patchy import random_patches
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = poe.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    gas = poe.biot_material(rho_f=100.0, k_f=0.02e9, eta=1e-5, **frame)
    ids = random_patches((NZ + 1, NX + 1), 0.5, fraction=0.2, r_min=1.0, r_max=4.0, seed=seed)
    return poe.coeffs_biot([water, gas], ids)


@pytest.mark.parametrize("fast", [False, True])
def test_palette_path_matches_planes_and_oracle(poe, oracle_mod, fast):
    """A two-material patchy model runs on the palette kernel (one byte per
    cell, TMA-staged tiles); the same model with palette=False reads its 8
    coefficient planes per cell (COEF).  Both must agree bit for bit, and with
    the oracle."""
    O = oracle_mod
    # 251 x 201 with a 10-cell C-PML: most 60 x 32 tiles are interior (no
    # edge, strip or source), the rest take the guarded path
    NX, NZ, dx, dt, f0, n = 250, 200, 0.5, 5e-5, 200.0, 140
    coef, vp = _patchy(poe, NX, NZ, 5)
    g = poe.grid(NX, NZ, dx, dt)
    px, pz = poe.pml_profiles(g, 10, f0, vp)
    rec = [(x, 15, c) for c in (0, 1, 2) for x in range(14, 240, 19)] + [(130, 100, 2), (95, 150, 1)]
    src = poe.source(64, 50, poe.SRC_RICKER_FZ, f0, 1e3, 0.0)
    out = {}
    for pal in (True, False):
        with poe.Solver(g, coef, px, pz, fast=fast, palette=pal) as s:
            s.add_shot(src, rec)
            s.run(n)
            out[pal] = (s.traces(), s.field("vz"), s.field("p"), s.field("sxx"))
    for a, b in zip(out[True], out[False]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    o = O.Oracle(O.F32 if fast else O.REFMIXED, NX, NZ, dx, dx, dt, coef, px, pz)
    o.set_source(64, 50, O.SRC_FZ, O.source_table(1, f0, dt, n, amplitude=1e3, t_cut=0.0, dx=dx, dz=dx))
    o.set_receivers(rec)
    ref = o.run(n)
    tol = TOL_FAST if fast else TOL_EXACT
    assert rel_l2(out[True][0], ref) <= tol
    r = o.field("vz")
    assert max_rel_peak(out[True][1], r, np.abs(r).max()) <= tol

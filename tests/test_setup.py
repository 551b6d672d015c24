"""Host-side set-up of the product library against the oracle and the golden
fixtures (bit-exact), plus C-ABI hygiene.  No GPU needed."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_library_exports_every_declared_symbol(poe):
    hdrs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]
    names = set()
    for h in hdrs:
        txt = open(h).read()
        names |= set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(poe_\w+)\s*\(", txt, flags=re.M))
    assert len(names) >= 20
    lib = poe.lib()
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_pml_matches_golden(poe):
    d = np.load(os.path.join(GOLD, "ref_setup.npz"))
    g = poe.grid(int(d["NX"]), int(d["NZ"]), float(d["dx"]), float(d["dt"]))
    px, pz = poe.pml_profiles(g, int(d["npml"]), float(d["f0"]), float(d["cp"].max()))
    assert bits_equal(px, d["prof_x"]) and bits_equal(pz, d["prof_z"])


@pytest.mark.parametrize("NX,NZ,dx,dt,npml,f0,cp", [
    (200, 200, 0.5, 5e-5, 20, 200.0, 3347.0),
    (2000, 2000, 0.5, 5e-5, 40, 200.0, 3400.0),
    (13599, 2439, 1.25, 95e-6, 10, 30.0, 4700.0),    # the reference's hard-coded grid (cu:486-510)
    (30, 17, 2.0, 1e-4, 9, 25.0, 3000.0),            # strips overlap
])
def test_pml_matches_oracle(poe, oracle_mod, NX, NZ, dx, dt, npml, f0, cp):
    g = poe.grid(NX, NZ, dx, dt)
    px, pz = poe.pml_profiles(g, npml, f0, cp)
    ox, oz = oracle_mod.pml_profiles(NX, NZ, dx, dx, dt, npml, cp, f0=f0)
    assert bits_equal(px, ox) and bits_equal(pz, oz)


def test_coeffs_from_medium_matches_golden(poe):
    d = np.load(os.path.join(GOLD, "ref_setup.npz"))
    g = poe.grid(int(d["NX"]), int(d["NZ"]), float(d["dx"]), float(d["dt"]))
    coef = poe.coeffs_from_medium(g, d["medium"], d["cp"], d["cs"], d["rho"])
    assert bits_equal(coef, d["coef"])


def test_coeffs_from_medium_rejects_unknown_id(poe):
    g = poe.grid(9, 9, 1.0, 1e-4)
    sh = (10, 10)
    med = np.zeros(sh, np.float32)
    med[3, 4] = 7.0
    with pytest.raises(poe.PoeError) as e:
        poe.coeffs_from_medium(g, med, np.full(sh, 3000.0), np.full(sh, 1500.0), np.full(sh, 2300.0))
    assert e.value.status == 1


def test_courant(poe):
    g = poe.grid(200, 200, 0.5, 5e-5)
    poe.check_courant(g, 3347.0)
    with pytest.raises(poe.PoeError) as e:
        poe.check_courant(g, 6100.0)    # 0.61 > (6/7)/sqrt(2)
    assert e.value.status == 2


@pytest.mark.parametrize("kind,amp,tcut,n", [(0, 1.0, 0.4, 9000), (1, 3.5, 0.0, 700), (1, 1.0, 0.01, 700)])
def test_source_tables_match_oracle(poe, oracle_mod, kind, amp, tcut, n):
    g = poe.grid(100, 80, 0.5, 5e-5)
    t1 = poe.source_table(g, poe.source(50, 40, kind, 200.0, amp, tcut), n)
    t2 = oracle_mod.source_table(kind, 200.0, 5e-5, n, amplitude=amp, t_cut=tcut, dx=0.5, dz=0.5)
    assert bits_equal(t1, t2)


def test_reference_source_cutoff_step(poe):
    # t = (n-1) dt as a float; the cut-off is t < 0.4 (cu:94, 107)
    g = poe.grid(100, 80, 1.25, 95e-6)
    t = poe.source_table(g, poe.source(50, 40, 0, 30.0), 10000)
    last = np.float32(np.float32(len(t) - 1) * np.float32(95e-6))
    nxt = np.float32(np.float32(len(t)) * np.float32(95e-6))
    assert float(last) < 0.4 <= float(nxt)


def test_ref_receivers(poe):
    g = poe.grid(66, 52, 1.25, 95e-6)
    r = poe.ref_receivers(g, 33, 26, 5, 6, 20, 30)
    assert r.shape == (2 * 5 + 2 * 6 + 4, 3)
    assert [tuple(x) for x in r[:5]] == [(33, 9, 1), (33, 19, 1), (33, 29, 1), (33, 39, 1), (33, 49, 1)]
    assert [tuple(x) for x in r[10:12]] == [(10, 10, 1), (21, 10, 1)]
    assert tuple(r[22]) == (32, 50, 1)        # y = 50 point
    g2 = poe.grid(40, 32, 1.25, 95e-6)
    r2 = poe.ref_receivers(g2, 20, 16, 4, 5, 12, 20)
    assert r2[2 * 4 + 2 * 5][2] == poe.REC_NONE   # y = 50 is outside a 33-row grid


def test_biot_config1_coefficients(poe):
    """Homogeneous water-saturated sandstone of the 201^2 single-shot case."""
    m = poe.biot_material(2650.0, 0.2, 37e9, 10e9, 8e9, 1000.0, 2.25e9, 1e-3, 1e-12, 2.0)
    coef, vp = poe.coeffs_biot([m], np.zeros((3, 4), np.uint8))
    c = coef[:, 0, 0]
    np.testing.assert_allclose(c, [2320.0, 1000.0, 1e4, 1e9, 9.826e9, 8e9, 0.7297, 9.689e9], rtol=2e-4)
    assert 3300.0 < vp < 3420.0
    assert np.all(coef == coef[:, :1, :1])


def test_biot_coefficients_match_oracle(poe, oracle_mod):
    """The oracle's restatement of the direct-Biot coefficients equals the
    library's bit for bit (planes and the dispersion-relation velocity): the
    CPU reference arm of the bench builds its inputs with it."""
    frame = dict(rho_s=2650.0, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    rng = np.random.default_rng(4)
    mats = [dict(phi=float(rng.uniform(0.1, 0.3)), rho_f=rf, k_f=kf, eta=eta, **frame)
            for rf, kf, eta in ((1000.0, 2.25e9, 1e-3), (100.0, 0.02e9, 1e-5), (700.0, 0.7e9, 0.03),
                                (1000.0, 2.25e9, 0.0))]
    ids = rng.integers(0, len(mats), (33, 47)).astype(np.uint8)
    coef, vp = poe.coeffs_biot([poe.biot_material(**m) for m in mats], ids)
    ocoef, ovp = oracle_mod.coeffs_biot(mats, ids)
    assert np.array_equal(coef.view(np.uint32), ocoef.view(np.uint32))
    assert np.float32(vp) == np.float32(ovp)


def _patchy_coef(poe, rng, shape, nmat):
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    mats = [poe.biot_material(rho_f=1000.0 - 900.0 * i / max(nmat - 1, 1), k_f=2.25e9 / (1 + 10 * i),
                              eta=1e-3 / (1 + i), **frame) for i in range(nmat)]
    ids = rng.integers(0, nmat, shape).astype(np.uint8)
    coef, _ = poe.coeffs_biot(mats, ids)
    return coef


@pytest.mark.parametrize("nmat", [1, 2, 17, 64])
def test_material_palette_matches_reference_float_ops(poe, nmat):
    """The palette poe_create builds: every cell's 8 coefficients come back
    bit for bit from its row, and the derived entries are the reference's
    per-cell float operations (cu:293-295, with the 0.50 double literal: a
    double sum of two floats rounded to float is the float sum, 53 >= 2*24+2)
    plus correctly rounded reciprocals."""
    rng = np.random.default_rng(nmat)
    dt = np.float32(5e-5)
    coef = _patchy_coef(poe, rng, (37, 53), nmat)
    pal = poe.material_palette(coef, dt)
    assert pal is not None
    ids, rows = pal
    assert rows.shape == (len(np.unique(ids)), 14) and rows.shape[0] == len(np.unique(coef.reshape(8, -1), axis=1).T)
    assert bits_equal(np.moveaxis(rows[ids][..., :8], -1, 0), coef)
    f = np.float32
    rho, rhof, rsm, eok = (rows[:, i] for i in range(4))
    co = (rho * rsm - rhof * rhof) / dt
    half = (rho * eok).astype(np.float64) * 0.50
    c1 = (co.astype(np.float64) + half).astype(f)
    c2 = (co.astype(np.float64) - half).astype(f)
    assert bits_equal(rows[:, 8], co) and bits_equal(rows[:, 9], c1) and bits_equal(rows[:, 10], c2)
    assert bits_equal(rows[:, 11], rhof * eok)
    assert bits_equal(rows[:, 12], (1.0 / co.astype(np.float64)).astype(f))
    assert bits_equal(rows[:, 13], (1.0 / c1.astype(np.float64)).astype(f))


def test_material_palette_declines_large_and_degenerate_models(poe):
    rng = np.random.default_rng(7)
    dt = 5e-5
    coef = _patchy_coef(poe, rng, (16, 16), 1)   # one material: density alone varies below
    coef65 = coef.copy()
    coef65[0] = (2000.0 + np.arange(256, dtype=np.float32) % 65).reshape(16, 16)   # 65 distinct densities
    assert poe.material_palette(coef65, dt) is None
    coef64 = coef.copy()
    coef64[0] = (2000.0 + np.arange(256, dtype=np.float32) % 64).reshape(16, 16)
    assert poe.material_palette(coef64, dt) is not None
    flat = coef.copy()
    flat[1] = 0.0
    flat[2] = 0.0                                # rho m - rho_f^2 = 0: co = 0 exactly
    assert poe.material_palette(flat, dt) is None
    with pytest.raises(poe.PoeError):
        poe.material_palette(coef, 0.0)

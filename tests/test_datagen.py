"""Synthetic workload generators: seeded, reproducible, with the statistics
the benchmark configurations ask for (CPU only)."""
import numpy as np

from poe2d_gb300 import datagen as D
from poe2d_gb300.patchy import random_patches, read_bin, reference_pattern, write_bin


def test_uneven_specs_ranges_and_determinism():
    a = D.uneven_specs(7, 256)
    assert a == D.uneven_specs(7, 256)
    side = np.array([s["side"] for s in a])
    assert side.min() >= 256 and side.max() <= 1536 and np.all([s["steps"] == 4 * s["side"] for s in a])
    for key, lo, hi in (("phi", 0.1, 0.3), ("gas", 0.0, 0.3), ("radius", 1.0, 10.0), ("f0", 150.0, 300.0)):
        v = np.array([s[key] for s in a])
        assert v.min() >= lo and v.max() <= hi
    n = D.uneven_specs(3, 16, 256, 256, 0.0, (0.2, 0.2), (150.0, 300.0))
    assert all(s["side"] == 256 and s["gas"] == 0.0 and s["phi"] == 0.2 for s in n)


def test_patchy_ids_reach_the_gas_fraction():
    for frac, r in ((0.1, 2.0), (0.3, 1.0), (0.05, 9.0)):
        ids = D.patchy_ids((400, 500), 0.5, frac, r, seed=5)
        assert ids.dtype == np.uint8 and set(np.unique(ids)) <= {0, 1}
        assert frac <= ids.mean() <= frac + 0.03
        assert np.array_equal(ids, D.patchy_ids((400, 500), 0.5, frac, r, seed=5))
    assert not D.patchy_ids((50, 50), 0.5, 0.0, 3.0, seed=1).any()


def test_random_patches_and_formats(tmp_path):
    ids = random_patches((120, 160), 0.5, fraction=0.1, r_min=2.0, r_max=10.0, seed=1234)
    assert 0.1 <= ids.mean() < 0.2
    for order in ("x", "z"):
        p = tmp_path / ("m_%s.bin" % order)
        write_bin(p, ids.astype(np.float32), order=order)
        assert p.stat().st_size == ids.size * 4
        back = read_bin(p, 160, 120, order=order)
        assert np.array_equal(back, ids.astype(np.float32))


def test_reference_patterns():
    for k in range(1, 7):
        m = reference_pattern(k)
        assert m.shape == (2800, 5000)
        assert set(np.unique(m[:2000])) == {1.0} and set(np.unique(m[2240:])) == {1.0}
        assert set(np.unique(m[2000:2240])) == {2.0, 3.0}
    # pattern 2 doubles pattern 1's lattice pitch: fewer circle cells
    assert (reference_pattern(2) == 2.0).sum() < (reference_pattern(1) == 2.0).sum()
    # exact circle-cell counts from the loop bounds of patchy:17-22 and 55-60
    # (r = 8: a disk sqrt(dx^2 + dy^2) <= r holds 197 cells):
    #   pattern 1, pitch 16: centres x = 9..4985 (312), z = 9..233 (15); tangent
    #     neighbours share one cell (15 x 311 across, 312 x 14 down); the last
    #     row loses its bottom cell to row 241 of the 240-row layer
    #   pattern 2, pitch 32: 156 x 8 disjoint disks, the last row clipped likewise
    assert (reference_pattern(1) == 2.0).sum() == 312 * 15 * 197 - 15 * 311 - 312 * 14 - 312
    assert (reference_pattern(2) == 2.0).sum() == 156 * 8 * 197 - 156


def test_resample_keeps_endpoints_and_linearity():
    t = np.stack([np.linspace(0, 1, 4000), np.sin(np.linspace(0, 3, 4000))], axis=1).astype(np.float32)
    r = D.resample(t, 1024)
    assert r.shape == (1024, 2)
    assert r[0, 0] == t[0, 0] and abs(r[-1, 0] - t[-1, 0]) < 1e-6
    assert np.allclose(r[:, 0], np.linspace(0, 1, 1024), atol=1e-6)


def test_surrogate_flop_count_matches_the_reference_layer_table():
    from oracle import surrogate_ref as R
    from poe2d_gb300.surrogate import forward_flops_per_sample
    rows = {"conv2d": lambda hw, up: (hw // 2) ** 2, "fc": lambda hw, up: 1, "conv1d": lambda hw, up: hw * up}
    flops = sum(2 * rows[k](hw, up) * R._k(k, ci) * co for k, ci, co, hw, up, _ in R.LAYERS)
    assert flops == forward_flops_per_sample()

"""The autotuner times the tile heights, work-list orders, graph lengths and
step-spanning launches on the context itself, keeps the fastest, and leaves
the shots at step 0; whatever it picks, the results equal the default
configuration's bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(poe):
    from poe2d_gb300.patchy import random_patches
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = poe.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    gas = poe.biot_material(rho_f=100.0, k_f=0.02e9, eta=1e-5, **frame)
    NX, NZ = 300, 200
    ids = random_patches((NZ + 1, NX + 1), 0.5, fraction=0.15, r_min=1.0, r_max=4.0, seed=21)
    coef, vp = poe.coeffs_biot([water, gas], ids)
    g = poe.grid(NX, NZ, 0.5, 5e-5)
    px, pz = poe.pml_profiles(g, 15, 200.0, vp)
    rec = [(x, 18, c) for c in (0, 1, 2) for x in range(20, 280, 17)]
    srcs = [poe.source(100 + 50 * k, 18, poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0) for k in range(3)]
    return g, coef, px, pz, rec, srcs


def _run(poe, m, tune):
    g, coef, px, pz, rec, srcs = m
    with poe.Solver(g, coef, px, pz, fast=True) as s:
        for src in srcs:
            s.add_shot(src, rec)
        picked = None
        if tune == "auto":
            picked = s.autotune(32) + (s.tuning(),)
            assert all(s.steps(k) == 0 for k in range(len(srcs)))
        elif tune is not None:
            s.tune(*tune[:2])
            if len(tune) > 2:
                s.tune_span(tune[2])
            if len(tune) > 3:
                s.tune_tile(tune[3])
            assert s.tuning() == dict(zip(("order", "graph_steps", "span", "tile_z"), tune + (2, 32)[len(tune) - 2:]))
        s.run(150)
        return [s.traces(k) for k in range(len(srcs))] + [s.field("vz", 2)], picked


def test_autotune_keeps_results_and_reports_timings(poe):
    m = _model(poe)
    ref, _ = _run(poe, m, None)
    got, (order, gsteps, ms, tuning) = _run(poe, m, "auto")
    assert order in (0, 1, 2, 3) and gsteps in (16, 64) and ms.shape == (32,)
    assert np.all(ms > 0)                     # FAST, no batch: every candidate runs, 16-row tiles too
    c = int(ms.argmin())
    assert ((c // 4) % 4, (16, 64)[(c // 2) % 2], c % 2, (32, 16)[c // 16]) == (
        order, gsteps, tuning["span"], tuning["tile_z"]) and tuning["order"] == order
    for a, b in zip(ref, got):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for tune in ((1, 16, 0), (2, 64, 1), (3, 64, 0, 16), (3, 16, 1, 16), (0, 64, 0), (0, 64, 1, 16),
                 (2, 16, 2, 16)):
        other, _ = _run(poe, m, tune)
        for a, b in zip(ref, other):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_tuning_arguments_are_checked(poe):
    g, coef, px, pz, rec, srcs = _model(poe)
    with poe.Solver(g, coef, px, pz) as s:
        s.add_shot(srcs[0], rec)
        with pytest.raises(poe.PoeError):
            s.tune(4, 64)
        with pytest.raises(poe.PoeError):
            s.tune(0, 0)
        with pytest.raises(poe.PoeError):
            s.tune_span(3)
        with pytest.raises(poe.PoeError):
            s.tune_tile(24)
        with pytest.raises(poe.PoeError):
            s.tune_tile(16)                   # EXACT stencils: 32-row tiles only
        assert s.tuning()["tile_z"] == 32
        s.run(5)
        with pytest.raises(poe.PoeError):
            s.autotune(8)                     # shots not at step 0


def test_span_auto_spans_steps_of_few_tiles_only(poe):
    """POE_SPAN_AUTO (the default): one spanning launch per 64-step graph for a
    step of at most 96 tiles per SM (one 1500 x 2000 shot, 1575 tiles, about
    10 per SM), one launch per step for a step of more (10 such shots, about
    104 per SM); SPAN_ALWAYS and SPAN_NEVER override it."""
    import torch
    assert poe.SPAN_AUTO == 2
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = poe.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    NX, NZ = 1499, 1999
    coef, vp = poe.coeffs_biot([water], np.zeros((NZ + 1, NX + 1), np.uint8))
    g = poe.grid(NX, NZ, 0.5, 5e-5)
    px, pz = poe.pml_profiles(g, 20, 200.0, vp)
    rec = [(x, 30, poe.REC_VZ) for x in range(100, 1400, 100)]
    tiles = -(-(NX + 1) // 60) * -(-(NZ + 1) // 32)
    for nshots, span, per_graph in ((1, None, 2), (10, None, 65), (10, poe.SPAN_ALWAYS, 2), (1, poe.SPAN_NEVER, 65)):
        assert (nshots * tiles <= 96 * sms) == (nshots == 1)
        with poe.Solver(g, coef, px, pz, fast=True) as s:
            for k in range(nshots):
                s.add_shot(poe.source(300 + 100 * k, 40, poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0), rec)
            if span is not None:
                s.tune_span(span)
            s.run(64)
            s.sync()
            n0 = s.launches
            s.run(128)
            s.sync()
            assert s.launches - n0 == 2 * per_graph, (nshots, span)


@pytest.mark.parametrize("palette", [True, False])
@pytest.mark.parametrize("kmax", [1.0, 1.5])
def test_small_tiles_equal_large_tiles(poe, palette, kmax):
    """60 x 16 tiles (FAST) end exactly where 60 x 32 tiles end, with and
    without step-spanning launches, K = 1 or not, palette or coefficient
    planes, through graphs, direct tails, a reset and a restored checkpoint;
    the batch takes 32-row contexts only."""
    g, coef, px, pz, rec, srcs = _model(poe)
    par = poe.pml_defaults(15, 200.0, 3000.0)
    par.k_max = kmax
    px, pz = poe.pml_profiles(g, params=par)
    out = []
    for tile, span in ((32, 0), (16, 0), (16, 1)):
        with poe.Solver(g, coef, px, pz, fast=True, palette=palette) as s:
            for src in srcs[:2]:
                s.add_shot(src, rec)
            s.tune_tile(tile)
            s.tune_span(span)
            s.run(150)
            img = s.checkpoint(1)
            s.run(40)
            s.reset_shot(0)
            s.run(70)
            s.restore(img, 1)
            s.run(33)
            out.append([(s.traces(k), s.field("vz", k), s.field("p", k), s.field("xi1", k)) for k in range(2)])
    for other in out[1:]:
        for a, b in zip(out[0], other):
            for x, y in zip(a, b):
                assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_batch_takes_large_tiles_only(poe):
    g, coef, px, pz, rec, srcs = _model(poe)
    a = poe.Solver(g, coef, px, pz, fast=True)
    b = poe.Solver(g, coef, px, pz, fast=True)
    for s in (a, b):
        s.add_shot(srcs[0], rec)
    a.tune_tile(16)
    with pytest.raises(poe.PoeError):
        poe.Batch([a, b])
    a.tune_tile(32)
    with poe.Batch([a, b]) as bt:
        with pytest.raises(poe.PoeError):
            b.tune_tile(16)                   # a batch member
        bt.run([10, 10])
        bt.sync()
    for s in (a, b):
        s.close()

"""Batched solver: several models of uneven sizes and step counts in one
persistent launch per step must end exactly where separate runs end.

The batch kernel is the step kernel over a concatenated work list
(model, shot, tile); each model reads its own grid, profiles and material
table (or coefficient planes), so the comparison with single-context runs
is bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _patchy(poe, NX, NZ, seed, phi=0.2):
    from poe2d_gb300.patchy import random_patches
    frame = dict(rho_s=2650.0, phi=phi, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = poe.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    gas = poe.biot_material(rho_f=100.0, k_f=0.02e9, eta=1e-5, **frame)
    ids = random_patches((NZ + 1, NX + 1), 0.5, fraction=0.2, r_min=1.0, r_max=4.0, seed=seed)
    return poe.coeffs_biot([water, gas], ids)


# (NX, NZ, npml, k_max, shots, f0): uneven sizes, one model with K != 1 in its C-PML
MODELS = [(130, 97, 10, 1.0, 2, 200.0), (251, 201, 12, 1.0, 1, 250.0), (77, 181, 8, 1.5, 1, 180.0),
          (190, 60, 6, 1.0, 2, 300.0), (300, 33, 5, 1.0, 1, 220.0)]


def _build(poe, fast):
    out = []
    for i, (NX, NZ, npml, kmax, nshots, f0) in enumerate(MODELS):
        coef, vp = _patchy(poe, NX, NZ, 40 + i, phi=0.15 + 0.03 * i)
        g = poe.grid(NX, NZ, 0.5, 5e-5)
        par = poe.pml_defaults(npml, f0, vp)
        par.k_max = kmax
        px, pz = poe.pml_profiles(g, params=par)
        rec = [(x, 3 + npml, c) for c in (0, 1, 2) for x in range(2, NX - 1, 11)] + [(NX // 2, NZ // 2, 2)]
        srcs = [poe.source(NX // 3 + 17 * s, npml + 4 + 5 * s, poe.SRC_RICKER_FZ if s == 0 else poe.SRC_REF_DGAUSS_P,
                           f0, 1e3 if s == 0 else 1.0, 0.0 if s == 0 else 0.4) for s in range(nshots)]
        out.append((g, coef, px, pz, srcs, rec))
    return out


def _solver(poe, case, fast, palette=True):
    g, coef, px, pz, srcs, rec = case
    s = poe.Solver(g, coef, px, pz, fast=fast, palette=palette)
    for src in srcs:
        s.add_shot(src, rec)
    return s


def _state(s, nshots):
    return [(s.traces(k), s.field("vz", k), s.field("p", k), s.field("wx", k), s.steps(k)) for k in range(nshots)]


def _same(a, b):
    for (ta, *fa, na), (tb, *fb, nb) in zip(a, b):
        assert na == nb
        assert np.array_equal(ta.view(np.uint32), tb.view(np.uint32))
        for x, y in zip(fa, fb):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("palette", [True, False])
@pytest.mark.parametrize("fast", [False, True])
@pytest.mark.parametrize("span", [1, 0])
def test_batch_matches_single_runs(poe, fast, palette, span):
    """The batch with step-spanning launches (span 1) or one launch per step
    (span 0) against single runs with the other setting."""
    cases = _build(poe, fast)
    runs = [[150, 70, 0, 213, 64], [40, 0, 100, 64, 1]]     # uneven, with idle models and graph + tail segments
    ref = [_solver(poe, c, fast, palette) for c in cases]
    for s in ref:
        s.tune_span(1 - span)
    for r in runs:
        for i, s in enumerate(ref):
            if r[i]:
                s.run(r[i])
    want = [_state(s, len(c[4])) for s, c in zip(ref, cases)]
    for s in ref:
        s.close()

    solvers = [_solver(poe, c, fast, palette) for c in cases]
    with poe.Batch(solvers) as b:
        b.tune_span(span)
        for r in runs:
            b.run(r)
        b.sync()
        assert b.launches > 0
    for s, c, w in zip(solvers, cases, want):
        _same(_state(s, len(c[4])), w)
    # a solver keeps running on its own after the batch
    solvers[1].run(33)
    assert solvers[1].steps() == 70 + 33
    for s in solvers:
        s.close()


def test_batch_rejects_mixed_contexts(poe):
    cases = _build(poe, False)[:2]
    a = _solver(poe, cases[0], False)
    b = _solver(poe, cases[1], True)
    with pytest.raises(poe.PoeError):
        poe.Batch([a, b])                     # mixed stencil modes
    g, coef, px, pz, srcs, rec = cases[1]
    c = poe.Solver(g, coef, px, pz, palette=False)
    c.add_shot(srcs[0], rec)
    with pytest.raises(poe.PoeError):
        poe.Batch([a, c])                     # a palette model with a per-cell coefficient model
    with pytest.raises(poe.PoeError):
        poe.Batch([a, a])                     # listed twice
    with poe.Batch([a]) as bt:
        with pytest.raises(poe.PoeError):
            bt.run([-1])
    for s in (a, b, c):
        s.close()


def test_batch_at_a_spacing_whose_24h_has_many_bits(poe):
    """h = 0.3: the batch launches the exact-division variant for any spacing;
    each model must end exactly where its own run ends."""
    cases = []
    for i, (NX, NZ) in enumerate([(90, 70), (130, 45)]):
        coef, vp = _patchy(poe, NX, NZ, 70 + i)
        g = poe.grid(NX, NZ, 0.3, 3e-5)
        px, pz = poe.pml_profiles(g, 8, 200.0, vp)
        rec = [(x, 12, c) for c in (0, 1, 2) for x in range(10, NX - 10, 9)]
        cases.append((g, coef, px, pz, [poe.source(NX // 2, 14, poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0)], rec))
    steps = [150, 97]
    ref = [_solver(poe, c, False) for c in cases]
    for s, n in zip(ref, steps):
        s.run(n)
    want = [_state(s, 1) for s in ref]
    solvers = [_solver(poe, c, False) for c in cases]
    with poe.Batch(solvers) as b:
        b.run(steps)
        b.sync()
    for s, w in zip(solvers, want):
        _same(_state(s, 1), w)
    for s in ref + solvers:
        s.close()


@pytest.mark.parametrize("fast", [False, True])
@pytest.mark.parametrize("palette", [True, False])
def test_step_spanning_launches_equal_one_launch_per_step(poe, fast, palette):
    """One context with several shots: step-spanning launches (a tile of step
    n starts once its neighbourhood has finished step n-1) end exactly where
    one launch per step ends, through graphs (64 steps), the direct tail, a
    single step, a reset and a restored checkpoint."""
    case = _build(poe, fast)[1][:4] + ([poe.source(60, 20, poe.SRC_RICKER_FZ, 250.0, 1e3, 0.0),
                                       poe.source(190, 40, poe.SRC_REF_DGAUSS_P, 250.0, 1.0, 0.4)],
                                      _build(poe, fast)[1][5])
    out = []
    for span in (0, 1):
        s = _solver(poe, case, fast, palette)
        s.tune_span(span)
        s.run(150)                         # two 64-step graphs and a 22-step direct launch
        s.run(1)
        img = s.checkpoint(1)
        s.run(63)
        s.reset_shot(0)
        s.run(70)                          # shot 0 from step 0 again, shot 1 on from 214
        s.restore(img, 1)                  # shot 1 back to step 151 (its tile flags go back too)
        s.run(40)
        out.append(_state(s, 2))
        s.close()
    _same(out[0], out[1])

"""Palette kernel at the edges of its geometry: grids smaller than one tile,
grids that are exact tile multiples (60 x 32 cells), the 64-material limit,
a C-PML with K != 1 on the single-model kernel, and sources next to the
grid's edges.  Each case must equal the same model read from its 8
coefficient planes (palette=False) bit for bit, and the oracle: bit for bit
with EXACT stencils, within 1e-5 relative L2 with FAST ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _materials(poe, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        out.append(poe.biot_material(rho_s=float(rng.uniform(2500, 2700)), phi=float(rng.uniform(0.1, 0.3)),
                                     k_s=37e9, k_frame=float(rng.uniform(8e9, 12e9)), mu_frame=float(rng.uniform(6e9, 9e9)),
                                     rho_f=float(rng.uniform(100, 1000)), k_f=float(rng.uniform(0.02e9, 2.25e9)),
                                     eta=1e-3, kappa=1e-12, tortuosity=2.0))
    return out


def _case(poe, oracle_mod, NX, NZ, nmat, kmax, src_xz, fast, n=90, seed=0, h=0.5):
    O = oracle_mod
    rng = np.random.default_rng(seed)
    ids = rng.integers(0, nmat, size=(NZ + 1, NX + 1)).astype(np.uint8)
    coef, vp = poe.coeffs_biot(_materials(poe, nmat, seed), ids)
    g = poe.grid(NX, NZ, h, 4e-5 * h / 0.5)
    par = poe.pml_defaults(min(8, NX // 4, NZ // 4), 200.0, vp)
    par.k_max = kmax
    px, pz = poe.pml_profiles(g, params=par)
    rec = [(x, z, c) for c in (0, 1, 2) for x in range(0, NX + 1, max(1, NX // 7)) for z in (0, NZ // 2, NZ)]
    src = poe.source(src_xz[0], src_xz[1], poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0)
    out = {}
    for pal in (True, False):
        with poe.Solver(g, coef, px, pz, fast=fast, palette=pal) as s:
            s.add_shot(src, rec)
            s.run(n)
            out[pal] = [s.traces(), s.field("vz"), s.field("p"), s.field("sxz")]
    for a, b in zip(out[True], out[False]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    o = O.Oracle(O.F32 if fast else O.REFMIXED, NX, NZ, g.dx, g.dz, g.dt, coef, px, pz)
    o.set_source(src_xz[0], src_xz[1], O.SRC_FZ, O.source_table(1, 200.0, g.dt, n, amplitude=1e3, t_cut=0.0,
                                                                  dx=g.dx, dz=g.dz))
    o.set_receivers(rec)
    ref = o.run(n)
    if not fast:   # EXACT: the oracle's mixed FP32/FP64 arithmetic, bit for bit
        assert np.array_equal(out[True][0].view(np.uint32), ref.view(np.uint32))
    tol = 1e-5 if fast else 1e-6
    ref = ref.astype(np.float64)
    assert np.abs(ref).max() > 0                # the source reached the receivers
    d = np.linalg.norm(out[True][0].astype(np.float64) - ref) / np.linalg.norm(ref)
    assert d <= tol, d


@pytest.mark.parametrize("fast", [False, True])
@pytest.mark.parametrize("NX,NZ,nmat,kmax,src", [
    (30, 20, 2, 1.0, (15, 10)),          # smaller than one 60 x 32 tile
    (119, 63, 5, 1.0, (60, 31)),         # exactly 2 x 2 tiles
    (179, 95, 64, 1.0, (90, 2)),         # the 64-material limit; source near the top edge
    (150, 90, 3, 1.7, (1, 45)),          # K != 1 in the C-PML; source on the first updated column
])
def test_palette_geometry_edges(poe, oracle_mod, fast, NX, NZ, nmat, kmax, src):
    _case(poe, oracle_mod, NX, NZ, nmat, kmax, src, fast)


def test_more_than_64_materials_use_the_planes(poe):
    rng = np.random.default_rng(1)
    ids = rng.integers(0, 65, size=(41, 61)).astype(np.uint8)
    ids.flat[:65] = np.arange(65)
    coef, vp = poe.coeffs_biot(_materials(poe, 65, 1), ids)
    g = poe.grid(60, 40, 0.5, 4e-5)
    px, pz = poe.pml_profiles(g, 8, 200.0, vp)
    with poe.Solver(g, coef, px, pz) as a, poe.Solver(g, coef, px, pz, palette=False) as b:
        for s in (a, b):
            s.add_shot(poe.source(30, 20, poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0), [(30, 10, 1)])
            s.run(40)
        assert np.array_equal(a.traces().view(np.uint32), b.traces().view(np.uint32))


@pytest.mark.parametrize("palette", [True, False])
def test_force_source_on_column_zero_excites_nothing(poe, palette):
    """The vz update starts at column 1 (cu:316-356), so a z-force on
    column 0 never enters the solution: every trace and field stays zero."""
    ids = np.zeros((61, 91), np.uint8)
    coef, vp = poe.coeffs_biot(_materials(poe, 1, 2), ids)
    g = poe.grid(90, 60, 0.5, 4e-5)
    px, pz = poe.pml_profiles(g, 8, 200.0, vp)
    with poe.Solver(g, coef, px, pz, palette=palette) as s:
        s.add_shot(poe.source(0, 30, poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0), [(x, 30, 1) for x in range(0, 91, 10)])
        s.run(60)
        assert not s.traces().any()
        assert not s.field("vz").any() and not s.field("p").any()


@pytest.mark.parametrize("h", [0.3, 0.1])
def test_exact_stencils_at_spacings_whose_24h_has_many_bits(poe, oracle_mod, h):
    """24 h = 7.2 or 2.4 (26 bits for 0.1): the stencil division keeps a float
    quotient only where its rounding is certain and takes the reference's FP64
    line elsewhere, so EXACT follows the oracle's FP64 stencils here too."""
    _case(poe, oracle_mod, 119, 63, 3, 1.0, (60, 31), False, h=h)

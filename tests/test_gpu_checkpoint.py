"""Full-state checkpoint / restart of a shot: a run that is saved, restored
(into a fresh context or the same one) and continued must equal the
uninterrupted run bit for bit, fields and traces."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(poe, palette):
    from poe2d_gb300.patchy import random_patches
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = poe.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    gas = poe.biot_material(rho_f=100.0, k_f=0.02e9, eta=1e-5, **frame)
    NX, NZ = 180, 140
    ids = random_patches((NZ + 1, NX + 1), 0.5, fraction=0.2, r_min=1.0, r_max=4.0, seed=9)
    coef, vp = poe.coeffs_biot([water, gas], ids)
    g = poe.grid(NX, NZ, 0.5, 5e-5)
    px, pz = poe.pml_profiles(g, 12, 200.0, vp)
    rec = [(x, 14, c) for c in (0, 1, 2) for x in range(15, 170, 13)]
    srcs = [poe.source(90, 20, poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0), poe.source(60, 70, poe.SRC_REF_DGAUSS_P, 250.0)]
    return g, coef, px, pz, rec, srcs


def _open(poe, m, palette):
    g, coef, px, pz, rec, srcs = m
    s = poe.Solver(g, coef, px, pz, palette=palette)
    for src in srcs:
        s.add_shot(src, rec)
    return s


FIELDS = ("vx", "vz", "wx", "wz", "sxz", "p", "sxx", "g11", "xi2")


def _snap(s, shot):
    return [s.traces(shot)] + [s.field(f, shot) for f in FIELDS]


def _eq(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert x.shape == y.shape and np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("palette", [True, False])
def test_restart_equals_uninterrupted_run(poe, palette):
    m = _model(poe, palette)
    a = _open(poe, m, palette)
    a.run(101)                                  # odd: the current buffer is the second one
    img = [a.checkpoint(k) for k in range(2)]
    a.run(77)
    want = [_snap(a, k) for k in range(2)]

    b = _open(poe, m, palette)                  # fresh context
    b.run(5)                                    # with stale state that the restore must replace
    for k in range(2):
        b.restore(img[k], k)
        assert b.steps(k) == 101
    b.run(77)
    for k in range(2):
        _eq(_snap(b, k), want[k])

    a.restore(img[1], 1)                        # back in time on the same context
    a.run(77)
    _eq(_snap(a, 1), want[1])
    a.close()
    b.close()


def test_checkpoint_rejects_mismatch_and_corruption(poe):
    m = _model(poe, True)
    a = _open(poe, m, True)
    a.run(40)
    img = a.checkpoint(0)
    with pytest.raises(poe.PoeError):
        a.restore(img, 1)                       # the other shot's source differs
    bad = bytearray(img)
    bad[len(bad) // 2] ^= 0x40
    with pytest.raises(poe.PoeError) as e:
        a.restore(bytes(bad), 0)
    assert e.value.status == 7                  # POE_EIO: checksum
    with pytest.raises(poe.PoeError):
        a.restore(img[:-4], 0)
    a.restore(img, 0)
    assert a.steps(0) == 40
    a.close()


def test_checkpoint_rejects_another_model_or_geometry(poe):
    """The header carries the spacings, the time step and hashes of the
    profiles, the coefficients and the receiver list: an image loads only
    into a shot of the same model and geometry, whatever the grid layout."""
    g, coef, px, pz, rec, srcs = m = _model(poe, True)
    a = _open(poe, m, True)
    a.run(30)
    img = a.checkpoint(0)
    info = poe.checkpoint_info(img)
    assert info["steps"] == 30 and info["nrec"] == len(rec) and info["dt"] == np.float32(5e-5)
    a.close()

    def refused(g2, coef2, px2, pz2, rec2, palette=True):
        s = poe.Solver(g2, coef2, px2, pz2, palette=palette)
        s.add_shot(srcs[0], rec2)
        with pytest.raises(poe.PoeError) as e:
            s.restore(img, 0)
        s.close()
        return e.value.status

    px2, pz2 = poe.pml_profiles(g, 12, 230.0, 3500.0)           # same strips, other damping
    assert px2.shape == px.shape and not np.array_equal(px2, px)
    assert refused(g, coef, px2, pz2, rec) == 1
    g2 = poe.grid(g.NX, g.NZ, g.dx, 4e-5)                        # another time step, same profiles
    assert refused(g2, coef, px, pz, rec) == 1
    coef2 = coef.copy()
    coef2[4, 70, 90] *= np.float32(1.0001)                       # one cell's lambda_c: a third material
    assert refused(g, coef2, px, pz, rec) == 1
    assert refused(g, coef2, px, pz, rec, palette=False) == 1
    rec2 = list(rec)
    rec2[5] = (rec2[5][0] + 1, rec2[5][1], rec2[5][2])          # one receiver moved by a cell
    assert refused(g, coef, px, pz, rec2) == 1


def test_checkpoint_moves_between_palette_and_planes(poe):
    """The coefficient hash is taken over the 8 planes, so an image saved by a
    context that keeps a material palette restores into one that keeps the
    planes (the same model), and the run goes on bit for bit."""
    m = _model(poe, True)
    a = _open(poe, m, True)
    a.run(64)
    img = a.checkpoint(1)
    a.run(40)
    want = _snap(a, 1)
    a.close()
    b = _open(poe, m, False)
    b.restore(img, 1)
    b.run(40)
    _eq(_snap(b, 1), want)
    b.close()

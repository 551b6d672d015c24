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

"""The kernels' waits are bounded: a wait whose phase never completes, or on a
tile flag that nothing sets, gives up, flags the error and ends its kernel,
and the device stays usable (no GPU is hung or faulted: the barrier simply
never receives an arrival, the flag is never written); the same flag wait on
flags that are set passes at once."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_waits_on_a_barrier_nobody_arrives_at_and_a_flag_nobody_sets_give_up(poe):
    assert poe.wait_limit_check(polls=1000)
    assert poe.wait_limit_check(polls=1)


def test_bad_poll_counts_are_rejected(poe):
    for polls in (0, -5, (1 << 24) + 1):
        with pytest.raises(poe.PoeError):
            poe.wait_limit_check(polls=polls)


def test_device_usable_after_a_wait_gave_up(poe):
    assert poe.wait_limit_check(polls=100)
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = poe.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    ids = np.zeros((61, 81), np.uint8)
    coef, vp = poe.coeffs_biot([water], ids)
    g = poe.grid(80, 60, 0.5, 5e-5)
    px, pz = poe.pml_profiles(g, 8, 200.0, vp)
    with poe.Solver(g, coef, px, pz) as s:
        s.add_shot(poe.source(40, 30, poe.SRC_RICKER_FZ, 200.0, 1e3, 0.0), [(40, 20, 1)])
        s.run(50)
        tr = s.traces()
    assert np.isfinite(tr).all() and np.abs(tr).max() > 0

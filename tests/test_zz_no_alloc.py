"""The allocation-free read-out of derived fields (collected last on purpose).

poe_get_derived_noalloc serves callers that cannot allocate device memory:
it builds sigma_xx, sigma_zz or p in the library's static scratch plane
instead of the buffer poe_get_field allocates.  Both read-outs run the same
arithmetic on the same state, so the output must equal poe_get_field's bit
for bit, on two calls in a row, through the C ABI.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(poe):
    from poe2d_gb300.patchy import random_patches
    frame = dict(rho_s=2650.0, phi=0.2, k_s=37e9, k_frame=10e9, mu_frame=8e9, kappa=1e-12, tortuosity=2.0)
    water = poe.biot_material(rho_f=1000.0, k_f=2.25e9, eta=1e-3, **frame)
    gas = poe.biot_material(rho_f=100.0, k_f=0.02e9, eta=1e-5, **frame)
    ids = random_patches((91, 121), 0.5, fraction=0.2, r_min=1.0, r_max=4.0, seed=9)
    return poe.coeffs_biot([water, gas], ids)


@pytest.mark.parametrize("palette", [True, False])
def test_noalloc_matches_get_field_twice(poe, palette):
    coef, vp = _model(poe)
    g = poe.grid(120, 90, 0.5, 5e-5)
    px, pz = poe.pml_profiles(g, 10, 200.0, vp)
    with poe.Solver(g, coef, px, pz, palette=palette) as s:
        s.add_shot(poe.source(60, 45, poe.SRC_REF_DGAUSS_P, 200.0, 1.0, 0.4), [(30, 20, 2)])
        s.run(90)
        for name in ("p", "sxx"):          # two calls in a row, different fields
            got = s.derived_noalloc(name)
            ref = s.field(name)
            assert np.abs(ref).max() > 0
            np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
        s.run(7)
        a, b = s.derived_noalloc("szz"), s.derived_noalloc("szz")
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
        np.testing.assert_array_equal(a.view(np.uint32), s.field("szz").view(np.uint32))
        with pytest.raises(poe.PoeError):
            s.derived_noalloc("vx")        # not a derived field

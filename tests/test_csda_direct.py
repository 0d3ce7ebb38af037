"""compute_flux_csda_direct (src/Geometry.jl:1126-1209), the closed-form
two-layer CSDA flux.  The reference's tests do not cover it, so the oracle is
checked against itself (dual-number derivative vs central differences;
closed form vs the adaptive CSDA walk of compute_flux_single), and the
device against the oracle."""
import math

import numpy as np
import pytest

CASES = [(100.0, 2650.0, 45.0), (500.0, 2400.0, 80.0), (30.0, 2800.0, 20.0)]


@pytest.fixture(scope="module")
def orc(oracle):
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR))


@pytest.mark.parametrize("thick,rho,elev", CASES)
def test_oracle_derivative_matches_finite_differences(oracle, orc, thick, rho, elev):
    for E in (3.0, 40.0, 900.0):
        f, d = oracle.flux_csda_direct(orc, 0, 1, rho, thick, elev, E, 1.0)
        h = 1e-3 * rho
        fp, _ = oracle.flux_csda_direct(orc, 0, 1, rho + h, thick, elev, E, 1.0)
        fm, _ = oracle.flux_csda_direct(orc, 0, 1, rho - h, thick, elev, E, 1.0)
        assert f > 0
        assert d == pytest.approx((fp - fm) / (2 * h), rel=1e-5)


def test_closed_form_tracks_adaptive_csda(oracle, orc):
    """The closed form and the stepped walk describe the same CSDA transport:
    for a 100 m column at 45 deg their fluxes agree to a few per cent (the
    walk evaluates the decay per step, the closed form at the layer mean)."""
    E = np.exp(np.linspace(np.log(20.0), np.log(1e3), 8))
    c, _ = oracle.backward_mc_csda(orc, 0, 1, 100.0, 2650.0, 45.0, E, np.ones(8), np.ones(8))
    for e, ci in zip(E, c):
        f, _ = oracle.flux_csda_direct(orc, 0, 1, 2650.0, 100.0, 45.0, e, 1.0)
        assert f == pytest.approx(ci, rel=0.03)


@pytest.mark.gpu
@pytest.mark.parametrize("thick,rho,elev", CASES)
def test_device_matches_oracle(oracle, orc, thick, rho, elev):
    import dpgpu
    phys = dpgpu.upload_physics([orc.table(0), orc.table(1)], ["StandardRock", "Air"])
    rng = np.random.default_rng(3)
    E = np.exp(rng.uniform(0.0, math.log(1e4), 256))
    q = np.where(rng.random(256) > 0.5, 1.0, -1.0)
    w = rng.uniform(0.5, 2.0, 256)
    c, d = dpgpu.csda_direct_samples(phys, E, q, w, rock_thickness=thick, rock_density=rho,
                                     elevation=elev)
    ref = np.array([oracle.flux_csda_direct(orc, 0, 1, rho, thick, elev, e, s) for e, s in zip(E, q)])
    np.testing.assert_allclose(c, w * ref[:, 0], rtol=1e-10, atol=0)
    np.testing.assert_allclose(d, w * ref[:, 1], rtol=1e-8, atol=1e-14 * np.abs(w * ref[:, 1]).max())
    f, g = dpgpu.compute_flux_gradient_csda(phys, rho, thick, elev, E[0], q[0])
    assert f == pytest.approx(ref[0, 0], rel=1e-12) and g == pytest.approx(ref[0, 1], rel=1e-10)

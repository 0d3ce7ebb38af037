"""CSDA -> MC correction calibration on the device water-fraction model
(calibrate_csda_correction, src/Tomography.jl:1061-1179;
calibrate_csda_material_correction, src/Tomography_material_calibration.jl):
the device calibration against the same calibration driven by the oracle's
model, and the reference's material test (test/test_tomography_material.jl)
run on the device."""
import math

import numpy as np
import pytest

from test_calibration import OracleModel, _calib_scene, _quadrature, _ref_path

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


@pytest.fixture(autouse=True)
def clean_corrections(dp):
    yield
    dp.set_csda_correction(enabled=False)
    dp.set_csda_material_correction(enabled=False)


@pytest.fixture(scope="module")
def orc40(oracle):
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), n=40,
                                  Kmin=1e-3, Kmax=1e6)


@pytest.fixture(scope="module")
def phys(dp, orc40):
    return dp.upload_physics([orc40.table(i) for i in range(3)], ["StandardRock", "Air", "Water"])


@pytest.mark.parametrize("fit_geometric", [True, False])
def test_device_calibration_matches_oracle_model(dp, phys, oracle, orc40, fit_geometric):
    """Noisy MC stand-ins (the corrected model at kappa_hard 17.3 with a
    geometric residual, times 2 % log-normal noise): the device calibration
    picks the oracle-driven calibration's kappa and residual."""
    mat = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    wf, paths = _calib_scene(dp, n=40, seed=5)
    samples = _quadrature(dp, 16, 1.0, 1e5)
    shallow = np.zeros(len(wf), bool)
    bins = list(range(1, len(paths) + 1))
    omodel = OracleModel(dp, oracle, orc40, mat, site, paths, samples, shallow)
    dp.set_csda_correction(enabled=True, kappa_strag=1.0, kappa_hard=17.3, resid_a=0.04,
                           resid_b=-0.01, resid_c=0.001, resid_d=0.05)
    mc = omodel.run(wf)[0] * np.exp(0.02 * np.random.default_rng(6).standard_normal(len(paths)))
    if not fit_geometric:
        dp.set_csda_correction(enabled=True, resid_a=0.03)
    kw = dict(fit_geometric=fit_geometric)
    keep = dp.get_csda_correction()
    ks, kh, st = dp.calibrate_csda_correction(phys, shallow, mat, site, paths, wf, samples, mc,
                                              bins, **kw)
    dev_corr = dp.get_csda_correction()
    dp.set_csda_correction(**keep._asdict())
    ks2, kh2, st2 = dp.calibrate_csda_correction(None, shallow, mat, site, paths, wf, samples, mc,
                                                 bins, model=omodel, **kw)
    assert (ks, kh) == (ks2, kh2)
    for k in ("resid_a", "resid_b", "resid_c", "resid_d"):
        assert st[k] == pytest.approx(st2[k], rel=1e-7, abs=1e-12)
    for k in ("rel_before", "rel_after", "mse_log"):
        assert st[k] == pytest.approx(st2[k], rel=1e-9)
    assert st["rel_after"] < st["rel_before"]
    assert dev_corr.kappa_hard == kh and dev_corr.resid_a == st["resid_a"]


def test_reference_material_test_on_device(dp):
    """test/test_tomography_material.jl:25-50 with the device model:
    create_physics(n_energies=40, K_min=0.001, K_max=1e6, [rock, air,
    water]); the on-path gradient against central differences (rtol 1e-4)
    and the synthetic contrast fit recovering (-0.7, 0.3) to 1e-9."""
    physics = dp.create_physics(n_energies=40, K_min=1e-3, K_max=1e6,
                                materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    idx = {n: i + 1 for n, i in physics.materials.items()}
    actual = dp.MaterialConfig(idx["StandardRock"], idx["Water"], idx["Air"], -1,
                               dp.STANDARD_ROCK.density, dp.WATER.density, 0.0, 0.0)
    site = dp.SiteConfig(1000.0, 12000.0)
    path, shallow, w = _ref_path(dp), [False, False], np.array([0.2, 0.4])
    samples = _quadrature(dp, 12, 1.0, 1e5)
    dp.set_csda_material_correction(linear=-0.7, quadratic=0.3)

    def full(x):
        return dp.compute_directional_flux_csda(physics, shallow, actual, site, path,
                                                np.asarray(x, np.float64), samples)

    fv, ids, grads = dp.directional_flux_and_grad_csda(physics, shallow, actual, site, path, w,
                                                       samples)
    assert fv == pytest.approx(full(w), rel=1e-14)
    h = 1e-6
    fd = [(full(w + h * (np.arange(2) == j - 1)) - full(w - h * (np.arange(2) == j - 1))) / (2 * h)
          for j in ids]
    np.testing.assert_allclose(grads, fd, rtol=1e-4)
    fields = [[0.1, 0.1], [0.5, 0.5], [0.8, 0.3]]
    base = np.zeros(2)
    m0 = [full(base)]
    mf = [[full(x)] for x in fields]
    fit = dp.calibrate_csda_material_correction(physics, shallow, actual, site, [path], base,
                                                fields, samples, m0, mf, [1], ridge=0.0)
    assert fit["linear"] == pytest.approx(-0.7, abs=1e-9)
    assert fit["quadratic"] == pytest.approx(0.3, abs=1e-9)
    assert fit["rms_log_after"] < 1e-12
    assert math.isfinite(fit["condition_number"])

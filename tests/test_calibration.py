"""CSDA -> MC correction calibration (src/Tomography.jl:1043-1179,
src/Tomography_material_calibration.jl) on the CPU: the host algebra of the
product's calibration driven by the oracle's water-fraction CSDA model in
place of the device batch, pinned to the reference's known answers
(test/test_tomography_material.jl)."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


@pytest.fixture(autouse=True)
def clean_corrections(dp):
    yield
    dp.set_csda_correction(enabled=False)
    dp.set_csda_material_correction(enabled=False)


class OracleModel:
    """The oracle's compute_directional_flux_csda over a list of paths, with
    the corrections in force at each call (the interface of CsdaBatch.run)."""

    def __init__(self, dp, oracle, orc_phys, matcfg, site, paths, samples, shallow):
        self.dp, self.o, self.p = dp, oracle, orc_phys
        self.cfg = [matcfg.rock_material - 1, matcfg.water_material - 1,
                    matcfg.air_material - 1,
                    matcfg.porous_material - 1 if matcfg.porous_material > 0 else -1]
        self.dens = [matcfg.rock_density, matcfg.water_density, matcfg.porous_density,
                     matcfg.porous_top_thickness]
        self.site = [site.detector_elevation, site.primary_altitude]
        self.paths, self.samples = paths, samples
        self.shallow = np.asarray(shallow, np.uint8)
        self.calls = 0

    def run(self, w, jacobian=False, precision="fp64"):
        self.calls += 1
        c, m = self.dp.get_csda_correction(), self.dp.get_csda_material_correction()
        corr = [int(c.enabled), c.kappa_strag, c.kappa_hard, c.resid_a, c.resid_b, c.resid_c,
                c.resid_d, int(m.enabled), m.linear, m.quadratic]
        P = self.paths
        seg_ptr = np.concatenate([[0], np.cumsum([len(p.segments) for p in P])])
        f = self.o.dir_csda(self.p, self.cfg, self.dens, self.site, corr,
                            [math.cos(math.radians(p.zenith)) for p in P],
                            [p.remaining_rock_distance for p in P],
                            [p.surface_exit_z for p in P], [int(p.valid) for p in P], seg_ptr,
                            [s.cell_idx - 1 for p in P for s in p.segments],
                            [s.distance for p in P for s in p.segments], self.shallow,
                            np.asarray(w, np.float64), [s.energy for s in self.samples],
                            [s.charge for s in self.samples], [s.weight for s in self.samples])
        return f, None


@pytest.fixture(scope="module")
def orc40(oracle):
    """create_physics(MUON; n_energies=40, K_min=0.001, K_max=1e6,
    materials=[STANDARD_ROCK, AIR, WATER])."""
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), n=40,
                                  Kmin=1e-3, Kmax=1e6)


def _quadrature(dp, n, lo, hi):
    """csda_energy_quadrature as EnergySample list (src/Tomography.jl:263-274)."""
    E, q, w = dp.csda_energy_quadrature(n, lo, hi)
    return [dp.EnergySample(*x) for x in zip(E, q, w)]


def _ref_path(dp):
    return dp.DirectionalPath(30.0, 0.0, [dp.CellSegment(1, 30.0), dp.CellSegment(2, 70.0)],
                              100.0, 200.0, 100.0, 0.0, True)


def test_material_multiplier_known_answer(dp):
    """test/test_tomography_material.jl:10-17: the column water fraction
    includes the dry remainder; zero water gives exactly 1."""
    mat = dp.MaterialConfig(1, 2, 3, -1, 2650.0, 1000.0, 0.0, 0.0)
    path, shallow, w = _ref_path(dp), [False, False], np.array([0.2, 0.4])
    dp.set_csda_material_correction(linear=-0.7, quadratic=0.3)
    gx = np.array([30.0, 70.0]) / ((1 - w) / 2650 + w / 1000)
    q = (w * gx).sum() / (gx.sum() + 100 * 2650)
    assert dp.column_water_fraction(mat, path, shallow, w) == pytest.approx(q, rel=1e-15)
    assert dp.csda_material_multiplier(path, shallow, mat, w) == pytest.approx(
        math.exp(-0.7 * q + 0.3 * q * q), rel=1e-15)
    assert dp.csda_material_multiplier(path, shallow, mat, np.zeros(2)) == 1.0
    dp.set_csda_material_correction(enabled=False)
    assert dp.csda_material_multiplier(path, shallow, mat, w) == 1.0
    with pytest.raises(ValueError):
        dp.set_csda_material_correction(linear=math.nan)


def test_material_calibration_recovers_synthetic_coefficients(dp, oracle, orc40):
    """test/test_tomography_material.jl:43-50: MC stand-ins generated by the
    CSDA model with (linear, quadratic) = (-0.7, 0.3); the unridged fit
    recovers them to 1e-9 and explains the contrasts to 1e-12."""
    mat = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(1000.0, 12000.0)
    path, shallow = _ref_path(dp), [False, False]
    samples = _quadrature(dp, 12, 1.0, 1e5)
    model = OracleModel(dp, oracle, orc40, mat, site, [path], samples, shallow)
    fields = [[0.1, 0.1], [0.5, 0.5], [0.8, 0.3]]
    base = np.zeros(2)
    dp.set_csda_material_correction(linear=-0.7, quadratic=0.3)
    m0 = [model.run(base)[0][0]]
    mf = [[model.run(np.array(x))[0][0]] for x in fields]
    fit = dp.calibrate_csda_material_correction(None, shallow, mat, site, [path], base, fields,
                                                samples, m0, mf, [1], ridge=0.0, model=model)
    assert fit["linear"] == pytest.approx(-0.7, abs=1e-9)
    assert fit["quadratic"] == pytest.approx(0.3, abs=1e-9)
    assert fit["rms_log_after"] < 1e-12
    assert fit["n_pairs"] == 3 and fit["n_fields"] == 3
    c = dp.get_csda_material_correction()
    assert c.enabled and c.linear == fit["linear"] and c.quadratic == fit["quadratic"]


def test_material_calibration_argument_errors_restore_state(dp):
    """The reference's ArgumentError / DimensionMismatch checks; a failed fit
    leaves the previous material correction installed."""
    mat = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(1000.0, 12000.0)
    path, shallow = _ref_path(dp), [False, False]
    dp.set_csda_material_correction(linear=0.25, quadratic=-0.5)
    args = (None, shallow, mat, site, [path], np.zeros(2))
    with pytest.raises(ValueError, match="two material training fields"):
        dp.calibrate_csda_material_correction(*args, [[0.1, 0.1]], [], [1.0], [[1.0]], [1])
    with pytest.raises(ValueError, match="matrix"):
        dp.calibrate_csda_material_correction(*args, [[0.1, 0.1], [0.2, 0.2]], [], [1.0],
                                              [[1.0, 1.0]], [1])
    with pytest.raises(ValueError, match="outside"):
        dp.calibrate_csda_material_correction(*args, [[0.1, 1.5], [0.2, 0.2]], [], [1.0],
                                              [[1.0], [1.0]], [1])

    class Broken:
        def run(self, w, jacobian=False, precision="fp64"):
            return np.array([-1.0]), None

    with pytest.raises(ValueError, match="invalid baseline flux"):
        dp.calibrate_csda_material_correction(*args, [[0.1, 0.1], [0.2, 0.2]], [], [1.0],
                                              [[1.0], [1.0]], [1], model=Broken())
    c = dp.get_csda_material_correction()
    assert c.enabled and (c.linear, c.quadratic) == (0.25, -0.5)


def test_corrections_artifact_round_trip(dp, tmp_path):
    """test/test_tomography_material.jl:51-58: the TOML artifact restores both
    corrections and returns the provenance; unsupported schemas and nonfinite
    coefficients are rejected before anything is installed."""
    dp.set_csda_correction(enabled=True, kappa_strag=1.0, kappa_hard=12.5, resid_a=0.1,
                           resid_b=-0.02, resid_c=0.003, resid_d=0.4)
    dp.set_csda_material_correction(linear=-0.7, quadratic=0.3)
    art = str(tmp_path / "corr.toml")
    dp.save_csda_corrections(art, metadata={"training_seeds": [12, 34], "source_hash": "fixture"})
    dp.set_csda_correction(enabled=False)
    dp.set_csda_material_correction(enabled=False)
    meta = dp.load_csda_corrections(art)
    assert meta["training_seeds"] == [12, 34] and meta["source_hash"] == "fixture"
    m = dp.get_csda_material_correction()
    assert m.enabled and m.linear == pytest.approx(-0.7, abs=1e-9) and m.quadratic == 0.3
    c = dp.get_csda_correction()
    assert c.enabled and (c.kappa_hard, c.resid_c, c.resid_d) == (12.5, 0.003, 0.4)
    text = open(art).read()
    with open(art, "w") as f:
        f.write(text.replace("schema_version = 1", "schema_version = 2"))
    with pytest.raises(ValueError, match="schema"):
        dp.load_csda_corrections(art)
    with open(art, "w") as f:
        f.write(text.replace("linear = -0.7", "linear = nan"))
    dp.set_csda_material_correction(linear=0.5, quadratic=0.5)
    with pytest.raises(ValueError, match="nonfinite"):
        dp.load_csda_corrections(art)
    assert dp.get_csda_material_correction().linear == 0.5


def _calib_scene(dp, n=24, seed=3):
    rng = np.random.default_rng(seed)
    n_cells = 12
    wf = rng.uniform(0.0, 0.3, n_cells)
    paths = []
    for _ in range(n):
        k = int(rng.integers(1, 6))
        segs = [dp.CellSegment(int(c), float(rng.uniform(5.0, 60.0)))
                for c in rng.integers(1, n_cells + 1, k)]
        paths.append(dp.DirectionalPath(float(rng.uniform(0.0, 65.0)), 0.0, segs, 0.0, 0.0,
                                        float(rng.uniform(20.0, 600.0)),
                                        float(rng.uniform(40.0, 300.0)), True))
    return wf, paths


def test_hard_loss_calibration_recovers_kappa(dp, oracle, orc40):
    """calibrate_csda_correction on MC stand-ins made by the corrected CSDA
    model with kappa_hard = 23.25 (a point of the refinement lattice) and no
    geometric residual: the grid search returns 23.25, the residual fit
    returns ~0 and the corrected flux matches the stand-ins; 'before' is
    the plain CSDA misfit.  Evaluations: 41 + 4 x 9 grid points, the
    'before', residual and 'after' passes."""
    mat = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    wf, paths = _calib_scene(dp)
    samples = _quadrature(dp, 16, 1.0, 1e5)
    shallow = np.zeros(len(wf), bool)
    bins = list(range(2, len(paths) + 1, 2))
    model = OracleModel(dp, oracle, orc40, mat, site, [paths[b - 1] for b in bins], samples,
                        shallow)
    dp.set_csda_correction(enabled=True, kappa_strag=1.0, kappa_hard=23.25)
    mc = model.run(wf)[0]
    dp.set_csda_correction(enabled=False)
    model.calls = 0
    ks, kh, st = dp.calibrate_csda_correction(None, shallow, mat, site, paths, wf, samples, mc,
                                              bins, model=model)
    assert ks == 1.0 and kh == 23.25
    assert model.calls == 41 + 4 * 9 + 3
    assert st["mse_log"] < 1e-24 and st["rel_after"] < 1e-12 and st["rel_before"] > 1e-3
    assert max(abs(st[k]) for k in ("resid_a", "resid_b", "resid_c", "resid_d")) < 1e-10
    c = dp.get_csda_correction()
    assert c.enabled and c.kappa_hard == 23.25


def test_geometric_residual_fit_and_frozen_mode(dp, oracle, orc40):
    """The ridged geometric fit: stand-ins with kappa_hard 10 and a residual
    exp(a + b logL + c logL^2 + d cos zenith); with ridge 0 the least-squares
    step reproduces the residual of the chosen kappa exactly, so the
    corrected model matches the stand-ins better than kappa alone.  With
    fit_geometric=False the installed residual is held during the search
    and kept."""
    mat = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    wf, paths = _calib_scene(dp, n=30, seed=4)
    samples = _quadrature(dp, 16, 1.0, 1e5)
    shallow = np.zeros(len(wf), bool)
    bins = list(range(1, len(paths) + 1))
    model = OracleModel(dp, oracle, orc40, mat, site, paths, samples, shallow)
    resid = dict(resid_a=0.05, resid_b=-0.01, resid_c=0.002, resid_d=0.03)
    dp.set_csda_correction(enabled=True, kappa_strag=1.0, kappa_hard=10.0, **resid)
    mc = model.run(wf)[0]
    # frozen residual: the search sees the true residual and finds kappa exactly
    ks, kh, st = dp.calibrate_csda_correction(None, shallow, mat, site, paths, wf, samples, mc,
                                              bins, fit_geometric=False, model=model)
    assert kh == 10.0 and st["rel_after"] < 1e-12
    assert all(st[k] == v for k, v in resid.items())
    # fitted residual: the least-squares step removes what kappa cannot
    dp.set_csda_correction(enabled=False)
    ks, kh, st = dp.calibrate_csda_correction(None, shallow, mat, site, paths, wf, samples, mc,
                                              bins, ridge_geom=0.0, model=model)
    c = dp.get_csda_correction()
    assert c.kappa_hard == kh and c.resid_a == st["resid_a"]
    dp.set_csda_correction(enabled=True, kappa_strag=1.0, kappa_hard=kh)
    f_kappa_only = model.run(wf)[0]
    rel_kappa_only = np.mean(np.abs(1 - f_kappa_only / mc))
    assert st["rel_after"] < rel_kappa_only
    # ridge anchoring pulls kappa toward the anchor
    _, kh_anchored, _ = dp.calibrate_csda_correction(
        None, shallow, mat, site, paths, wf, samples, mc, bins, fit_geometric=False,
        kh_anchor=40.0, kh_anchor_weight=10.0, model=model)
    assert kh_anchored > kh


def test_calibration_rejects_missing_reference_fluxes(dp):
    mat = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    with pytest.raises(RuntimeError, match="no positive MC reference fluxes"):
        dp.calibrate_csda_correction(None, [False], mat, dp.SiteConfig(963.0, 3e4), [], [0.0], [],
                                     [0.0, math.nan], [1, 2], model=object())
    with pytest.raises(ValueError):
        dp.calibrate_csda_correction(None, [False], mat, dp.SiteConfig(963.0, 3e4), [], [0.0], [],
                                     [1.0], [1, 2], model=object())

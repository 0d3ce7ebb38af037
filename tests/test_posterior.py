"""Posterior and fit statistics of src/Tomography_inverse.jl:895-1127:
the reference's own checks (test/test_tomography.jl:336-371,
test/stability_v2.jl:12-22 and 49-51), the Huber prior's local curvature
against finite differences, and (GPU) the statistics over the device
water-fraction operator against the same statistics over the oracle's
model."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


def _fd_jacobian(f, w, h=1e-6):
    w = np.asarray(w, np.float64)
    cols = []
    for k in range(len(w)):
        e = np.zeros(len(w))
        e[k] = h
        cols.append((np.asarray(f(w + e)) - np.asarray(f(w - e))) / (2 * h))
    return np.column_stack(cols)


def test_reference_posterior_null_and_profile(dp):
    """test/test_tomography.jl:336-371 (section 9): n = 6 cells, m = 40 rows
    of |N(0,1)| + 0.2 (numpy's generator stands in for Julia's seed 7)."""
    rng = np.random.default_rng(7)
    n, m = 6, 40
    A = np.abs(rng.standard_normal((m, n))) + 0.2
    wtrue = np.array([0.0, 0.4, 0.0, 0.6, 0.1, 0.0])
    free = np.ones(n, bool)
    import scipy.sparse as sp

    def lin(w):
        return A @ w, sp.csr_matrix(A)

    Wv = np.full(m, 50.0)
    post = dp.laplace_posterior(lin, wtrue, weights=Wv,
                                prior=dp.SmoothnessPrior([[] for _ in range(n)], 0.0), free=free)
    cov = np.linalg.inv(A.T @ np.diag(Wv) @ A)
    np.testing.assert_allclose(post["sigma"], np.sqrt(np.diag(cov)), rtol=1e-5)
    assert post["p_eff"] == pytest.approx(float(n), abs=1e-5)
    post_s = dp.laplace_posterior(lin, wtrue, weights=Wv,
                                  prior=dp.SmoothnessPrior([[(i + 1) % n] for i in range(n)], 5.0),
                                  free=free)
    assert post_s["p_eff"] < post["p_eff"]
    nz = post["sigma"] > 0
    np.testing.assert_allclose(post["z"][nz], wtrue[nz] / post["sigma"][nz], rtol=1e-14)
    np.testing.assert_allclose(post["resolution"], 1.0, atol=1e-5)

    def f(w):
        return np.exp(-(A @ np.asarray(w)))

    meas = f(wtrue)
    fitm, wdem, expo = np.ones(m), np.ones(m), 1e8
    nulls = dp.null_model_tests(f, wtrue, 0.3, free, meas, fitm, wdem, expo, p_eff=post["p_eff"])
    assert nulls["chi2_fit"] < nulls["chi2_dry"]
    assert nulls["chi2_fit"] < nulls["chi2_unif"]
    assert nulls["sigma_dry"] > 3.0
    assert nulls["aic"]["fit"] < nulls["aic"]["dry"]
    assert nulls["ndata"] == m

    prof = dp.profile_inventory(f, wtrue, free, meas, fitm, wdem, expo, n_grid=41)
    assert prof["T_map"] == pytest.approx(wtrue.sum(), rel=1e-9)
    assert np.all(prof["dchi2"] >= -1e-9)
    assert abs(prof["T"][np.argmin(prof["chi2"])] - wtrue.sum()) < 0.2 * wtrue.sum()
    assert len(prof["T"]) == 41


def test_posterior_free_set_and_edge_curvature(dp):
    """Cells outside free report zero; the Huber prior's posterior curvature
    (src/Tomography_inverse.jl:282-293) equals the finite-difference Hessian
    of prior_value where no edge difference sits at a knot, and drops the
    edges beyond delta."""
    from dpgpu.inverse import prior_value
    from dpgpu.posterior import _prior_posterior_hessian
    rng = np.random.default_rng(3)
    n = 7
    nb = [[(i + 1) % n, (i + 3) % n] for i in range(n)]
    prior = dp.EdgePrior(nb, 0.8, 0.15)
    w = rng.uniform(0.0, 0.6, n)
    H = _prior_posterior_hessian(prior, w)
    h = 1e-4
    num = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            ei, ej = np.eye(n)[i] * h, np.eye(n)[j] * h
            num[i, j] = (prior_value(prior, w + ei + ej) - prior_value(prior, w + ei - ej) -
                         prior_value(prior, w - ei + ej) + prior_value(prior, w - ei - ej)) / (4 * h * h)
    np.testing.assert_allclose(H, num, atol=1e-6)
    diffs = [abs(w[i] - w[j]) for i, nbi in enumerate(prior.neighbors) for j in nbi if i < j]
    assert any(d > prior.delta for d in diffs) and any(d <= prior.delta for d in diffs)

    A = np.abs(rng.standard_normal((20, n))) + 0.1
    free = np.array([1, 0, 1, 1, 0, 1, 1], bool)
    post = dp.laplace_posterior(lambda x: (A @ x, A), w, weights=np.full(20, 3.0), prior=prior,
                                free=free)
    assert np.all(post["sigma"][~free] == 0) and np.all(post["resolution"][~free] == 0)
    lam = post["JtWJ"] + post["HR"]
    idx = np.nonzero(free)[0]
    lff = lam[np.ix_(idx, idx)]
    rg = 1e-9 * (np.trace(lff) / len(idx) + 1.0)
    cov = np.linalg.inv(lff + rg * np.eye(len(idx)))
    np.testing.assert_allclose(post["sigma"][idx], np.sqrt(np.diag(cov)), rtol=1e-12)
    assert post["p_eff"] == pytest.approx(np.trace(cov @ post["JtWJ"][np.ix_(idx, idx)]),
                                          rel=1e-12)


def test_chi2_sigma_and_profile_crossings(dp):
    """Wilson-Hilferty (src/Tomography_inverse.jl:963-969) and the crossing
    interpolation of profile_inventory: each reported crossing lies where
    the piecewise-linear calibrated residual increase equals 1."""
    from dpgpu.posterior import _chi2_sigma
    assert _chi2_sigma(5.0, 0.0) == 0.0
    k = 4.0
    assert _chi2_sigma(k * (1 - 2 / (9 * k)) ** 3, k) == pytest.approx(0.0, abs=1e-12)
    assert _chi2_sigma(30.0, 2.0) > 3.0
    # pred = 1 + w (one bin per cell), meas at the unit amplitude; the
    # normalisation is refit at every amplitude
    w_map = np.array([0.2, 0.3, 0.0])
    meas = np.array([1.2, 1.3, 1.0])
    fitm = np.array([1.0, 1.0, 1.0])

    def f(w):
        return 1.0 + np.asarray(w)

    prof = dp.profile_inventory(f, w_map, np.array([1, 1, 0], bool), meas, fitm, np.ones(3), 1e4,
                                n_grid=29, span=(0.2, 3.0))
    cal = prof["dchi2_cal"]
    kmin = int(np.argmin(prof["chi2"]))
    lo, hi = prof["ci68"]
    for x in (lo, hi):
        if math.isfinite(x):
            k = np.searchsorted(prof["w_mean"], x) - 1
            t = (x - prof["w_mean"][k]) / (prof["w_mean"][k + 1] - prof["w_mean"][k])
            assert cal[k] + t * (cal[k + 1] - cal[k]) == pytest.approx(1.0, rel=1e-9)
    assert math.isfinite(hi) and hi > prof["w_mean"][kmin]
    lo95, hi95 = prof["ci95"]
    assert hi95 > hi


def test_reference_profiled_log_operator(dp):
    """test/stability_v2.jl:12-22: the operator's Jacobian against central
    differences (rtol 1e-6, atol 1e-8), scale at the truth = 2.5, invalid
    arguments rejected; with weights and a pinned normalisation too."""
    A = np.array([[1.0, 0.2], [-0.3, 1.0], [0.6, -0.7], [-0.8, -0.1]])

    def model(w):
        p = np.exp(A @ w)
        return p, p[:, None] * A

    observed = np.exp(A @ np.array([0.3, 0.6])) * 2.5
    robust, scale = dp.profiled_log_observation_operator(model, observed, robust_scale=0.3)
    with pytest.raises(ValueError):
        dp.profiled_log_observation_operator(model, observed, normalization=-1)
    with pytest.raises(ValueError):
        dp.profiled_log_observation_operator(model, observed, robust_scale=math.inf)
    with pytest.raises(ValueError):
        dp.profiled_log_observation_operator(model, -observed)
    with pytest.raises(ValueError):
        dp.profiled_log_observation_operator(model, observed, weights=[1.0, 2.0])
    w = np.array([0.1, 0.4])
    r, J = robust(w)
    fd = _fd_jacobian(lambda x: robust(x)[0], w)
    np.testing.assert_allclose(J, fd, rtol=1e-6, atol=1e-8)
    assert scale(model(np.array([0.3, 0.6]))[0]) == pytest.approx(2.5, rel=1e-12)
    # the robust objective is sum r^2 / 2 = sum W c^2 (h - 1) (pseudo-Huber)
    z = np.log(model(w)[0]) - np.log(observed) + math.log(scale(model(w)[0]))
    hh = np.sqrt(1 + (z / 0.3) ** 2)
    assert 0.5 * float(r @ r) == pytest.approx(float(np.sum(0.09 * (hh - 1))), rel=1e-12)

    wts = np.array([1.0, 0.5, 0.8, 2.0])
    for norm in (0.0, 1.7):
        op, _ = dp.profiled_log_observation_operator(model, observed, weights=wts,
                                                     robust_scale=0.3, normalization=norm)
        r2, J2 = op(w)
        np.testing.assert_allclose(J2, _fd_jacobian(lambda x: op(x)[0], w), rtol=1e-6, atol=1e-8)


def test_reference_predict_only_residual(dp):
    """test/stability_v2.jl:43-51: the cheap residual path equals the
    operator's residual and calls only the prediction callback."""
    calls, cheap = [0], [0]

    def model(w):
        calls[0] += 1
        return np.array([math.exp(w[0] ** 3)]), np.array([[3 * w[0] ** 2 * math.exp(w[0] ** 3)]])

    def prediction(w):
        cheap[0] += 1
        return np.array([math.exp(w[0] ** 3)])

    op, _, predict = dp.profiled_log_observation_operator(
        model, [math.exp(0.125)], normalization=1.0, robust_scale=0.3, predict_only=prediction,
        return_predict_only=True)
    for w in ([0.01], [0.2], [0.5], [0.9]):
        c0 = calls[0]
        res = predict(np.array(w))
        assert calls[0] == c0
        assert np.array_equal(res, op(np.array(w))[0])
    assert cheap[0] == 4


@pytest.mark.gpu
def test_statistics_over_the_device_operator(dp, oracle):
    """The statistics over make_csda_operator (the device water-fraction
    flux and Jacobian) against the same statistics over the oracle's flux
    with a central-difference Jacobian: posterior sigma and p_eff, the
    robust operator's Jacobian, and the null-model residuals.  The
    derivative tolerance is the reference's own for its on-path gradient
    against central differences (rtol 1e-4, test/test_tomography_material.jl):
    the tables are piecewise interpolants, so a difference step that crosses
    a node carries an O(h) error."""
    from test_calibration import OracleModel, _calib_scene, _quadrature
    orc = oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), n=40,
                                 Kmin=1e-3, Kmax=1e6)
    phys = dp.upload_physics([orc.table(i) for i in range(3)], ["StandardRock", "Air", "Water"])
    mat = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    wf, paths = _calib_scene(dp, n=40, seed=5)
    samples = _quadrature(dp, 16, 1.0, 1e5)
    shallow = np.zeros(len(wf), bool)
    model = dp.make_csda_operator(phys, shallow, mat, site, paths, samples, n_cells=len(wf),
                                  valid_bins=list(range(len(paths))))
    omodel = OracleModel(dp, oracle, orc, mat, site, paths, samples, shallow)

    def oflux(w):
        return np.asarray(omodel.run(np.asarray(w, np.float64))[0])

    def omodel_fd(w):
        return oflux(w), _fd_jacobian(oflux, w)

    pred, J = model(wf)
    np.testing.assert_allclose(pred, oflux(wf), rtol=1e-10)
    seen = np.asarray(abs(J).sum(0)).ravel() > 0
    W = 1.0 / (0.02 * pred) ** 2
    prior = dp.SmoothnessPrior([[k + 1] if k + 1 < len(wf) else [] for k in range(len(wf))], 1e-3)
    post = dp.laplace_posterior(model, wf, weights=W, prior=prior, free=seen)
    opost = dp.laplace_posterior(omodel_fd, wf, weights=W, prior=prior, free=seen)
    np.testing.assert_allclose(post["sigma"], opost["sigma"], rtol=1e-4)
    assert post["p_eff"] == pytest.approx(opost["p_eff"], rel=1e-4)
    assert 0 < post["p_eff"] <= seen.sum() + 1e-9

    obs = oflux(np.clip(wf * 1.3, 0, 0.9)) * 1.7
    op, scale = dp.profiled_log_observation_operator(model, obs, weights=np.ones(len(obs)),
                                                     robust_scale=0.3)
    r, Jr = op(wf)
    fd = _fd_jacobian(lambda x: op(x)[0], wf)
    np.testing.assert_allclose(Jr, fd, rtol=1e-4, atol=1e-6)
    assert scale(oflux(np.clip(wf * 1.3, 0, 0.9))) == pytest.approx(1.7, rel=1e-9)

    def dflux(w):
        return model(np.asarray(w, np.float64))[0]

    fitm, wdem = np.ones(len(obs)), np.ones(len(obs))
    nd = dp.null_model_tests(dflux, wf, 0.2, seen, obs, fitm, wdem, 1e6, p_eff=post["p_eff"])
    no = dp.null_model_tests(oflux, wf, 0.2, seen, obs, fitm, wdem, 1e6, p_eff=post["p_eff"])
    for k in ("chi2_dry", "chi2_unif", "chi2_fit"):
        assert nd[k] == pytest.approx(no[k], rel=1e-9)

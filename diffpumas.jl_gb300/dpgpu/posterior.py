"""Posterior and fit statistics of src/Tomography_inverse.jl:895-1127 over a
forward model.

The model is the same closure the solvers take: model(w) -> (pred, J), J
dense or scipy-sparse (`make_csda_operator` gives the device water-fraction
flux and its Jacobian from one launch).  What follows the model call is small
dense algebra on the host, as in the reference: the Laplace posterior on the
free cells, the weighted-residual comparisons with the dry and uniform
fields, the amplitude scan of the inventory, and the pseudo-Huber log-ratio
residual operator with its profiled normalisation.
"""
import math

import numpy as np

from .inverse import EdgePrior, MAX_WATER_FRACTION, _prior_hessian


def _dense(J):
    return J.toarray() if hasattr(J, "toarray") else np.asarray(J, np.float64)


def _prior_posterior_hessian(prior, w):
    """The prior's local curvature at w (src/Tomography_inverse.jl:281-293):
    the smoothness prior's exact quadratic Laplacian; for the Huber prior the
    true second derivative (weight on the edges whose difference lies within
    delta, the interior side at a knot), not the IRLS majoriser."""
    n = len(w)
    if not isinstance(prior, EdgePrior):
        return _prior_hessian(prior, w).toarray()
    H = np.zeros((n, n))
    if prior.delta > 0:
        for i, nb in enumerate(prior.neighbors):
            for j in nb:
                if i < j and abs(w[i] - w[j]) <= prior.delta:
                    H[i, i] += prior.weight
                    H[j, j] += prior.weight
                    H[i, j] -= prior.weight
                    H[j, i] -= prior.weight
    return H


def laplace_posterior(model, w, *, weights, prior=None, free, ridge=1e-9):
    """Gaussian-linear posterior at the MAP field w (src/Tomography_inverse.jl:917-946).

    Precision Lambda = J^T W J + H_R, inverted on the free cells with the
    ridge ridge * (tr(Lambda_ff)/|free| + 1).  Returns a dict with sigma
    (per-cell posterior standard deviation), z = w / sigma and resolution
    (diagonal of Sigma_ff J^T W J_ff), zero outside free; p_eff (trace of the
    resolution matrix), JtWJ and HR."""
    w = np.asarray(w, np.float64)
    _, J = model(w)
    J = _dense(J)
    W = np.asarray(weights, np.float64)
    JtWJ = J.T @ (W[:, None] * J)
    HR = np.zeros_like(JtWJ) if prior is None else _prior_posterior_hessian(prior, w)
    lam = JtWJ + HR
    n = len(w)
    idx = np.nonzero(np.asarray(free, bool))[0]
    sigma, z, res, p_eff = np.zeros(n), np.zeros(n), np.zeros(n), 0.0
    if len(idx):
        lff = lam[np.ix_(idx, idx)]
        rg = ridge * (np.trace(lff) / len(idx) + 1.0)
        m = lff + rg * np.eye(len(idx))
        m = np.triu(m) + np.triu(m, 1).T  # Symmetric(...): the upper triangle
        cov = np.linalg.inv(m)
        rff = cov @ JtWJ[np.ix_(idx, idx)]
        p_eff = float(np.trace(rff))
        sigma[idx] = np.sqrt(np.maximum(np.diag(cov), 0.0))
        pos = sigma[idx] > 0
        z[idx[pos]] = w[idx[pos]] / sigma[idx[pos]]
        res[idx] = np.diag(rff)
    return {"sigma": sigma, "z": z, "p_eff": p_eff, "resolution": res, "JtWJ": JtWJ, "HR": HR}


def _weighted_chi2(flux_only, w, meas, fit_mask, wdem, exposure):
    """Weighted residual of a field with the log-scale s refit to it
    (src/Tomography_inverse.jl:950-959): (chi2, s)."""
    pred = np.asarray(flux_only(w), np.float64)
    meas = np.asarray(meas, np.float64)
    fm = np.asarray(fit_mask, np.float64)
    mw = fm.sum()
    s = math.exp(float(np.sum(fm * (np.log(np.maximum(meas, 1e-300)) -
                                    np.log(np.maximum(pred, 1e-300))))) / max(mw, 1e-30))
    obs = meas / s
    var = np.maximum(obs, 0.0) / exposure
    Wv = fm * np.asarray(wdem, np.float64) / np.maximum(var, 1e-300)
    return float(np.sum(Wv * (pred - obs) ** 2)), s


def _chi2_sigma(chi2, k):
    """Wilson-Hilferty Gaussian sigma of chi2 with k degrees of freedom
    (src/Tomography_inverse.jl:963-969); 0 for k <= 0."""
    if k <= 0:
        return 0.0
    t = (chi2 / k) ** (1.0 / 3.0)
    return (t - (1.0 - 2.0 / (9.0 * k))) / math.sqrt(2.0 / (9.0 * k))


def null_model_tests(flux_only, w_map, w0_uniform, free, meas, fit_mask, wdem, exposure, *, p_eff):
    """Weighted-residual comparison of the fit with dry rock and a uniform
    field on the free cells (src/Tomography_inverse.jl:983-1008).  The sigma,
    aic and bic entries are the reference's heuristic scores, kept by name."""
    w_map = np.asarray(w_map, np.float64)
    free = np.asarray(free, bool)
    w_dry = np.zeros(len(w_map))
    w_unif = np.where(free, float(w0_uniform), 0.0)
    c_dry, _ = _weighted_chi2(flux_only, w_dry, meas, fit_mask, wdem, exposure)
    c_unif, _ = _weighted_chi2(flux_only, w_unif, meas, fit_mask, wdem, exposure)
    c_fit, _ = _weighted_chi2(flux_only, w_map, meas, fit_mask, wdem, exposure)
    ndata = int(np.count_nonzero(np.asarray(fit_mask, np.float64) > 0.0))
    var_scale = max(c_fit / max(ndata - p_eff, 1.0), 1e-30)
    d_dry, d_unif = c_dry - c_fit, c_unif - c_fit
    dp_dry, dp_unif = max(p_eff, 1e-6), max(p_eff - 1.0, 1e-6)

    def aic(c, p):
        return c / var_scale + 2 * p

    def bic(c, p):
        return c / var_scale + p * math.log(max(ndata, 1))

    return {"chi2_dry": c_dry, "chi2_unif": c_unif, "chi2_fit": c_fit, "ndata": ndata,
            "var_scale": var_scale, "dchi2_dry": d_dry, "dchi2_unif": d_unif, "p_eff": p_eff,
            "sigma_dry": _chi2_sigma(max(d_dry, 0.0) / var_scale, dp_dry),
            "sigma_unif": _chi2_sigma(max(d_unif, 0.0) / var_scale, dp_unif),
            "aic": {"dry": aic(c_dry, 0.0), "unif": aic(c_unif, 1.0), "fit": aic(c_fit, p_eff)},
            "bic": {"dry": bic(c_dry, 0.0), "unif": bic(c_unif, 1.0), "fit": bic(c_fit, p_eff)}}


def profile_inventory(flux_only, w_map, free, meas, fit_mask, wdem, exposure, *, var_scale=1.0,
                      n_grid=21, span=(0.2, 3.0), w_max=MAX_WATER_FRACTION):
    """Amplitude scan of the weighted residual (src/Tomography_inverse.jl:1029-1069):
    the fitted field times each of n_grid amplitudes over span, clipped to
    [0, w_max], with the normalisation refit at each point.  ci68 / ci95 are
    the interpolated crossings of the calibrated residual increase at 1 and
    3.84 on each side of the minimum, in mean-water units (NaN when the grid
    holds no crossing)."""
    w_map = np.asarray(w_map, np.float64)
    nfree = max(int(np.count_nonzero(np.asarray(free, bool))), 1)
    Ts, wbar, chis = [], [], []
    for sc in np.linspace(span[0], span[1], n_grid):
        w = np.clip(sc * w_map, 0.0, w_max)
        T = float(w.sum())
        c, _ = _weighted_chi2(flux_only, w, meas, fit_mask, wdem, exposure)
        Ts.append(T)
        wbar.append(T / nfree)
        chis.append(c)
    Ts, wbar, chis = np.array(Ts), np.array(wbar), np.array(chis)
    kmin = int(np.argmin(chis))
    dchi = chis - chis[kmin]
    cal = dchi / max(var_scale, 1e-30)

    def crossings(thr):
        lo = hi = math.nan
        for k in range(kmin, 0, -1):
            if cal[k] <= thr <= cal[k - 1]:
                f = (thr - cal[k]) / (cal[k - 1] - cal[k] + 1e-30)
                lo = wbar[k] + f * (wbar[k - 1] - wbar[k])
                break
        for k in range(kmin, len(cal) - 1):
            if cal[k] <= thr <= cal[k + 1]:
                f = (thr - cal[k]) / (cal[k + 1] - cal[k] + 1e-30)
                hi = wbar[k] + f * (wbar[k + 1] - wbar[k])
                break
        return lo, hi

    return {"T": Ts, "w_mean": wbar, "chi2": chis, "dchi2": dchi, "dchi2_cal": cal,
            "T_map": float(w_map.sum()), "T_min": float(Ts[kmin]), "w_mean_min": float(wbar[kmin]),
            "ci68": crossings(1.0), "ci95": crossings(3.84), "var_scale": var_scale}


def profiled_log_observation_operator(model, observed, *, weights=None, robust_scale=1.0,
                                      normalization=0.0, predict_only=None,
                                      return_predict_only=False):
    """Pseudo-Huber residual operator on log flux ratios
    (src/Tomography_inverse.jl:1081-1127).

    t = log(pred) - log(observed) + a with a = log(normalization) when
    normalization > 0, else the root of sum W (t / sqrt(1 + (t/c)^2)) = 0 found
    by 80 bisections.  operator(w) -> (residual, Jacobian) with residual =
    sqrt(W) t sqrt(2 / (h + 1)), h = sqrt(1 + (t/c)^2), and the exact Jacobian
    including the implicit derivative of a; scale(pred) -> exp(a).  With
    return_predict_only, a third callable gives the residual alone (through
    predict_only(w) when given, else the model).  Invalid arguments raise
    ValueError (the reference's ArgumentError / DimensionMismatch)."""
    observed = np.asarray(observed, np.float64)
    if not np.all(np.isfinite(observed) & (observed > 0)):
        raise ValueError("log observations must be finite and positive")
    W = np.ones(len(observed)) if weights is None else np.asarray(weights, np.float64)
    if len(W) != len(observed):
        raise ValueError("weights must match observations")
    if not (math.isfinite(normalization) and normalization >= 0):
        raise ValueError("normalization must be finite and nonnegative")
    c = float(robust_scale)
    if not (math.isfinite(c) and c > 0):
        raise ValueError("robust_scale must be positive")
    if not (np.all(np.isfinite(W) & (W >= 0)) and W.sum() > 0):
        raise ValueError("weights must be nonnegative with positive sum")
    logobs = np.log(observed)
    sw = np.sqrt(W)

    def transform(pred):
        pred = np.asarray(pred, np.float64)
        if len(pred) != len(observed):
            raise ValueError("prediction must match observations")
        if not np.all(np.isfinite(pred) & (pred > 0)):
            raise ValueError("log predictions must be finite and positive")
        z = np.log(pred) - logobs
        a = math.log(normalization) if normalization > 0 else 0.0
        if normalization <= 0:
            lo, hi = -float(z.max()), -float(z.min())
            for _ in range(80):
                a = (lo + hi) / 2
                u = z + a
                score = float(np.sum(W * (u / np.sqrt(1 + (u / c) ** 2))))
                if score > 0:
                    hi = a
                else:
                    lo = a
            a = (lo + hi) / 2
        t = z + a
        h = np.sqrt(1 + (t / c) ** 2)
        residual = sw * t * np.sqrt(2 / (h + 1))  # rationalised: no cancellation near 0
        derivative = sw / h * np.sqrt((h + 1) / 2)
        return residual, derivative, h, math.exp(a), pred

    def operator(w):
        pred, J = model(w)
        residual, derivative, h, _, pred = transform(pred)
        D = _dense(J) / pred[:, None]
        if normalization <= 0:
            curvature = W / h ** 3
            D = D - (curvature @ D) / curvature.sum()
        return residual, derivative[:, None] * D

    def scale(pred):
        return transform(pred)[3]

    def residual_only(w):
        pred = model(w)[0] if predict_only is None else predict_only(w)
        return transform(pred)[0]

    if return_predict_only:
        return operator, scale, residual_only
    return operator, scale

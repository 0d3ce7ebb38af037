"""The inverse solvers of src/Tomography_inverse.jl (host algorithms over a
sparse Jacobian): single iterations against their update formulas, priors
against finite differences, Gauss-Newton on a linear model (CPU only), and
on the device water-fraction operator (GPU)."""
import math

import numpy as np
import pytest
import scipy.sparse as sp


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


def _system(seed=0, m=40, n=12):
    rng = np.random.default_rng(seed)
    A = sp.random(m, n, density=0.3, random_state=rng, format="csr") + sp.eye(m, n, format="csr")
    w_true = rng.uniform(0.05, 0.5, n)
    return A.tocsr(), w_true, A @ w_true


def _chain(n):
    return [[k - 1] if k else [] for k in range(n)]  # each cell linked to the previous one


def test_sart_iteration(dp):
    A, _, b = _system()
    w0 = np.full(A.shape[1], 0.2)
    w, h = dp.sart_reconstruct(A, b, w0=w0, n_iter=1, relaxation=0.3)
    Ad = A.toarray()
    rows = np.abs(Ad).sum(1)
    cols = np.abs(Ad).sum(0)
    ref = np.clip(w0 + 0.3 * (Ad.T @ ((b - Ad @ w0) / rows)) / cols, 0.0, 0.9)
    np.testing.assert_allclose(w, ref, rtol=1e-14)
    assert h[0] == pytest.approx(np.linalg.norm(b - Ad @ ref))


def test_mlem_iteration_with_prior(dp):
    A, _, b = _system(1)
    n = A.shape[1]
    prior = dp.SmoothnessPrior(_chain(n), 0.05)
    w0 = np.full(n, 0.3)
    w, _ = dp.mlem_reconstruct(A, b, w0=w0, n_iter=1, prior=prior)
    Ad = A.toarray()
    denom = Ad.sum(0) + np.maximum(dp.laplacian_gradient(prior, w0), 0.0)
    ref = np.clip(w0 * (Ad.T @ (b / np.maximum(Ad @ w0, 1e-12))) / denom, 0.0, 0.9)
    np.testing.assert_allclose(w, ref, rtol=1e-14)


def test_priors_match_finite_differences(dp):
    rng = np.random.default_rng(2)
    n = 10
    w = rng.uniform(0.0, 0.6, n)
    nb = [[(k + 1) % n, (k + 3) % n] for k in range(n)]
    for prior, grad in ((dp.SmoothnessPrior(nb, 0.7), dp.laplacian_gradient),
                        (dp.EdgePrior(nb, 0.7, 0.05), dp.edge_gradient)):
        g = grad(prior, w)
        for k in range(n):
            e = np.zeros(n)
            e[k] = 1e-6
            fd = (dp.prior_value(prior, w + e) - dp.prior_value(prior, w - e)) / 2e-6
            assert g[k] == pytest.approx(fd, rel=1e-6, abs=1e-9)
    # the smoothness prior's Gauss-Newton curvature is its exact Hessian 2 weight L
    prior = dp.SmoothnessPrior(nb, 0.7)
    H = dp.edge_hessian(dp.EdgePrior(prior.neighbors, 1.4, math.inf), w).toarray()
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1e-4
        col = (dp.laplacian_gradient(prior, w + e) - dp.laplacian_gradient(prior, w - e)) / 2e-4
        np.testing.assert_allclose(H[:, k], col, atol=1e-9)
    with pytest.raises(ValueError):
        dp.SmoothnessPrior([[5]], 1.0)


def test_gradient_descent_first_steps(dp):
    A, _, b = _system(3)
    model = lambda w: (A @ w, A)
    w0 = np.full(A.shape[1], 0.2)
    g = A.T @ (A @ w0 - b)
    w, _ = dp.gradient_descent_reconstruct(model, b, w0=w0, n_iter=1, lr=0.01, optimizer="adam")
    np.testing.assert_allclose(w, np.clip(w0 - 0.01 * g / (np.abs(g) + 1e-8), 0, 0.9), rtol=1e-12)
    w, _ = dp.gradient_descent_reconstruct(model, b, w0=w0, n_iter=1, lr=1.0, optimizer="pgd")
    d = np.asarray(A.multiply(A).sum(0)).ravel()
    p = g / np.maximum(d, 1e-9 * d.max())
    Ap = A @ p
    alpha = min(max((g @ p) / (Ap @ Ap), 0.0), 1.0)
    np.testing.assert_allclose(w, np.clip(w0 - alpha * p, 0, 0.9), rtol=1e-12)


def test_gauss_newton_recovers_linear_model(dp):
    A, w_true, b = _system(4)
    model = lambda w: (A @ w, A)
    stop = [None]
    w, h = dp.gauss_newton_reconstruct(model, b, w0=np.full(A.shape[1], 0.45), n_iter=8,
                                       lm_damping=1e-6, stop=stop)
    np.testing.assert_allclose(w, w_true, atol=1e-6)
    assert h[-1] < 1e-6 * h[0]
    assert dp.rmse(w, w_true) < 1e-6


@pytest.mark.gpu
def test_gauss_newton_on_the_device_operator(dp):
    """make_csda_operator (src/Tomography_inverse.jl:614-626) on the
    water-fraction kernel: noise-free data of a truth field on a coarse grid
    (4x4x4 cells of 160 m seen by 256 directions, an overdetermined problem);
    Gauss-Newton lowers the misfit and the error of the seen cells."""
    from dpgpu.workloads import directional_config
    phys = dp.create_physics(materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    raw, wf = directional_config(256, nx=4, ny=4, nz=4, pitch=160.0, seed=5)
    paths = [dp.DirectionalPath(z, a, [dp.CellSegment(c, l) for c, l in segs], tin, slant, rem,
                                sz, True) for z, a, segs, tin, slant, rem, sz in raw]
    site = dp.SiteConfig(963.0, 30000.0)
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2710.0, 1000.0, 0.0, 0.0)
    nodes = [dp.EnergySample(*x) for x in zip(*dp.csda_energy_quadrature(16, 1.0, 1e6))]
    n = len(wf)
    sh = np.zeros(n, bool)
    model = dp.make_csda_operator(phys, sh, cfg, site, paths, nodes, n_cells=n,
                                  valid_bins=list(range(len(paths))))
    obs, J = model(wf)
    assert J.shape == (len(paths), n)
    # the reference's normal equations are dense: solve for the cells the rays see
    seen = np.asarray(abs(J).sum(0)).ravel() > 0
    w0 = np.full(n, 0.15)
    w, h = dp.gauss_newton_reconstruct(model, obs, w0=w0, n_iter=3, free=seen)
    assert h[-1] < 0.5 * h[0]
    assert dp.rmse(w, wf, seen) < dp.rmse(w0, wf, seen)
    assert np.array_equal(w[~seen], w0[~seen])

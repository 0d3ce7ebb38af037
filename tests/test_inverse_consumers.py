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


# ---------------------------------------------------------------- the reference's
# known answers (test/test_inverse_solver.jl:4-112), graphs 0-based here
def test_prior_graph_and_curvature(dp):
    graph = [[1, 1, 0], [], [1]]
    smooth = dp.SmoothnessPrior(graph, 2.3)
    assert smooth.neighbors == [[1], [0, 2], [1]]
    edge = dp.EdgePrior(graph, 2.3, 0.2)
    assert edge.neighbors == smooth.neighbors
    w, h = np.array([0.1, 0.4, 0.8]), 1e-6
    from dpgpu.inverse import _prior_hessian
    for prior, grad in ((smooth, dp.laplacian_gradient), (edge, dp.edge_gradient)):
        fd = [(dp.prior_value(prior, w + h * e) - dp.prior_value(prior, w - h * e)) / (2 * h)
              for e in np.eye(3)]
        np.testing.assert_allclose(grad(prior, w), fd, rtol=1e-8, atol=1e-9)
    H = _prior_hessian(smooth, w).toarray()
    Hfd = np.column_stack([(dp.laplacian_gradient(smooth, w + h * e) -
                            dp.laplacian_gradient(smooth, w - h * e)) / (2 * h) for e in np.eye(3)])
    np.testing.assert_allclose(H, Hfd, rtol=1e-8, atol=1e-9)
    np.testing.assert_allclose(H @ np.ones(3), 0.0, atol=1e-12)
    assert np.linalg.eigvalsh(H).min() >= -1e-10
    # Julia's array isapprox is norm-wise: an exact 0 matches a last-bit residue
    np.testing.assert_allclose(_prior_hessian(edge, w) @ w, dp.edge_gradient(edge, w), atol=1e-12)


def _identity(v):
    return np.array(v, float), sp.identity(len(v), format="csr")


def test_gauss_newton_known_answers(dp):
    # from a perfect data fit the prior still moves the field to the MAP point
    prior = dp.SmoothnessPrior([[1], [0]], 10.0)
    fit, hist = dp.gauss_newton_reconstruct(_identity, [1.0, 0.0], w0=[1.0, 0.0], prior=prior,
                                            n_iter=12, box=(0.0, 1.0))
    np.testing.assert_allclose(fit, [21 / 41, 20 / 41], atol=1e-6)
    assert np.linalg.norm(fit - [1.0, 0.0]) > 0.1
    assert 0.5 * np.linalg.norm(fit - [1.0, 0.0]) ** 2 + dp.prior_value(prior, fit) < \
        dp.prior_value(prior, [1.0, 0.0])
    assert hist[0] == 0 and hist[-1] > 0
    # a fixed neighbour contributes curvature but does not move
    boundary = lambda v: (np.array([v[0]]), sp.csr_matrix([[1.0, 0.0]]))
    fixed, _ = dp.gauss_newton_reconstruct(boundary, [0.0], w0=[0.1, 0.8],
                                           prior=dp.SmoothnessPrior([[1], [0]], 2.0),
                                           free=[True, False], n_iter=12)
    assert fixed[1] == 0.8 and fixed[0] == pytest.approx(0.64, abs=1e-6)
    nonlinear = lambda v: (np.array([math.exp(v[0]) + 0.3 * v[1], 0.4 * v[0] + math.exp(v[1])]),
                           sp.csr_matrix([[math.exp(v[0]), 0.3], [0.4, math.exp(v[1])]]))
    fit, _ = dp.gauss_newton_reconstruct(nonlinear, [1.3, 1.6], w0=[0.1, 0.4], weights=[2.0, 5.0],
                                         prior=dp.SmoothnessPrior([[1], [0]], 0.7),
                                         free=[True, False], n_iter=30)
    assert fit[1] == 0.4 and fit[0] == pytest.approx(0.24287925833166624, abs=2e-6)
    # every coordinate fixed: one model call, the start returned
    calls = [0]

    def counted(v):
        calls[0] += 1
        return _identity(v)
    allfixed, allhist = dp.gauss_newton_reconstruct(counted, [0.0, 0.0], w0=[0.2, 0.8],
                                                    free=[False, False], n_iter=12)
    assert list(allfixed) == [0.2, 0.8] and len(allhist) == 1 and calls[0] == 1
    with pytest.raises(ValueError):
        dp.gauss_newton_reconstruct(_identity, np.zeros(2), w0=np.zeros(2), free=[True])
    # the affine tangent at w0 when not relinearising
    affine = lambda v: (np.array([2 + 3 * v[0]]), sp.csr_matrix([[3.0]]))
    frozen, _ = dp.gauss_newton_reconstruct(affine, [3.5], w0=[0.1], relinearize=False,
                                            n_iter=12)
    assert frozen[0] == pytest.approx(0.5, abs=1e-7)


def test_gradient_descent_known_answers(dp):
    calls = [0]

    def nonlinear(v):
        calls[0] += 1
        return np.array([2 + v[0] + v[0] ** 2]), sp.csr_matrix([[1 + 2 * v[0]]])
    gd, _ = dp.gradient_descent_reconstruct(nonlinear, [2.8], w0=[0.2], relinearize=False,
                                            optimizer="gd", n_iter=150, lr=0.1)
    assert gd[0] == pytest.approx(0.6, abs=1e-7) and calls[0] == 1
    step_model = lambda v: (np.array(v, float), sp.csr_matrix([[1.0]]))
    fit, h = dp.gradient_descent_reconstruct(step_model, [1.0], w0=[0.0], optimizer="gd",
                                             n_iter=1, lr=0.1)
    assert h[-1] == pytest.approx(np.linalg.norm(fit - [1.0]))
    flat_calls = [0]

    def flat(v):
        flat_calls[0] += 1
        return np.array([0.0]), sp.csr_matrix((1, 5))
    prior = dp.SmoothnessPrior([[1], [0, 2], [1, 3], [2, 4], [3]], 1.0)
    start = np.array([0.0, 0.1, 0.6, 0.3, 0.9])
    smoothed, _ = dp.gradient_descent_reconstruct(flat, [0.0], w0=start, prior=prior,
                                                  optimizer="pgd", n_iter=50, lr=1.0)
    assert flat_calls[0] > 3
    assert dp.prior_value(prior, smoothed) < 1e-6 * dp.prior_value(prior, start)
    affine = lambda v: (np.array([2 + 3 * v[0]]), sp.csr_matrix([[3.0]]))
    _, h = dp.gradient_descent_reconstruct(affine, [3.5], w0=[-2.0], optimizer="pgd", n_iter=4,
                                           lr=1.0)
    assert abs(h[-1]) < 1e-5


def test_gauss_newton_prediction_only_line_search(dp):
    """test/test_inverse_solver.jl:76-112."""
    target = np.array([math.exp(8 * 0.65)])
    counts = {"ref": 0, "fast": 0, "pred": 0}
    primal = lambda v: np.array([math.exp(8 * v[0])])

    def make(key):
        def model(v):
            counts[key] += 1
            return primal(v), sp.csr_matrix([[8 * math.exp(8 * v[0])]])
        return model

    def predict(v):
        counts["pred"] += 1
        return primal(v)
    full, fh = dp.gauss_newton_reconstruct(make("ref"), target, w0=[0.01], n_iter=20,
                                           box=(0.0, 1.0))
    cheap, ch = dp.gauss_newton_reconstruct(make("fast"), target, w0=[0.01], n_iter=20,
                                            box=(0.0, 1.0), predict_only=predict)
    np.testing.assert_allclose(cheap, full, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ch, fh, rtol=1e-12, atol=1e-12)
    assert cheap[0] == pytest.approx(0.65, abs=1e-8)
    assert counts["fast"] < counts["ref"] and counts["pred"] > 0
    # an inaccurate prediction may not authorise an objective increase
    checked, hist = dp.gauss_newton_reconstruct(make("fast"), target, w0=[0.01], n_iter=8,
                                                box=(0.0, 1.0), predict_only=lambda v: target)
    assert np.all(np.diff(hist) <= 1e-10)
    assert np.linalg.norm(primal(checked) - target) < np.linalg.norm(primal([0.01]) - target)
    zero_calls = [0]

    def zero_model(v):
        zero_calls[0] += 1
        return np.array(v, float), sp.csr_matrix([[1.0]])
    sat, hist = dp.gauss_newton_reconstruct(zero_model, [2.0], w0=[0.9], n_iter=8)
    assert list(sat) == [0.9] and zero_calls[0] == 1 and len(hist) == 2


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


# ---------------------------------------------- active-set mode (test/stability_v2.jl)
def test_reference_gn_acceptance_rule(dp):
    """test/stability_v2.jl:3-11: projection can turn a descent direction
    uphill at a shortened step; the active-set rule asks for descent and
    the Armijo decrease."""
    from dpgpu.inverse import _gn_accept_trial
    initial = np.array([0.1, 0.05, 0.9])
    direction = np.array([10.0, -10.0, -1.0])
    full = np.clip(initial + direction, 0.0, 1.0) - initial
    short = np.clip(initial + 0.05 * direction, 0.0, 1.0) - initial
    assert np.ones(3) @ full < 0 and np.ones(3) @ short > 0
    assert not _gn_accept_trial(1.00001, 1.0, np.ones(3), short, "active_set")
    assert not _gn_accept_trial(0.9, 1.0, np.ones(3), short, "active_set")
    assert _gn_accept_trial(0.9, 1.0, np.ones(3), full, "active_set")
    assert not _gn_accept_trial(math.nan, 1.0, np.ones(3), full, "legacy")
    with pytest.raises(ValueError):
        dp.gauss_newton_reconstruct(lambda w: (w, np.eye(1)), [0.0], w0=[0.1], solver_mode="x")


def _robust_example(dp):
    A = np.array([[1.0, 0.2], [-0.3, 1.0], [0.6, -0.7], [-0.8, -0.1]])

    def model(w):
        p = np.exp(A @ w)
        return p, p[:, None] * A

    observed = np.exp(A @ np.array([0.3, 0.6])) * 2.5
    return dp.profiled_log_observation_operator(model, observed, robust_scale=0.3)


@pytest.mark.parametrize("initial", [[0.0, 0.0], [0.7, 0.7], [0.1, 0.8]])
def test_reference_active_set_recovers_robust_fit(dp, initial):
    """test/stability_v2.jl:23-29: the robust log-ratio operator from three
    starting points converges to (0.3, 0.6) with a KKT residual below 1e-8
    and a non-increasing objective."""
    robust, _ = _robust_example(dp)
    diagnostics = []
    fit, _ = dp.gauss_newton_reconstruct(robust, np.zeros(4), w0=initial, n_iter=100,
                                         solver_mode="active_set", projected_gradient_tol=1e-9,
                                         diagnostics=diagnostics)
    np.testing.assert_allclose(fit, [0.3, 0.6], atol=1e-5)
    assert diagnostics[-1]["projected_gradient"] < 1e-8
    assert np.all(np.diff([d["objective"] for d in diagnostics]) <= 1e-12)


def test_reference_active_set_coupled_bound(dp):
    """test/stability_v2.jl:31-38: a coupled normal matrix where clipping
    the unconstrained Newton step stalls; the active set reaches the bound."""
    B = np.array([[1.0, 0.9], [0.0, 0.2]])
    diagnostics, stop = [], [None]
    fit, _ = dp.gauss_newton_reconstruct(lambda w: (B @ w, B), [-1.0, 0.4], w0=[0.0, 0.5],
                                         n_iter=100, solver_mode="active_set",
                                         diagnostics=diagnostics, projected_gradient_tol=1e-9,
                                         stop=stop)
    assert fit[0] == pytest.approx(0.0, abs=1e-8)
    assert diagnostics[-1]["projected_gradient"] < 1e-8
    assert stop == ["projected_gradient"]


def test_reference_cheap_residual_search(dp):
    """test/stability_v2.jl:41-66: line searches through the prediction
    callback give the same fit with fewer full-model calls; the bounded
    projected-gradient rescue recovers a cubic whose derivative vanishes at
    the start."""
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
    calls[0] = 0
    plain, _ = dp.gauss_newton_reconstruct(op, [0.0], w0=[0.01], n_iter=20,
                                           solver_mode="active_set")
    plain_calls = calls[0]
    calls[0] = cheap[0] = 0
    events, log, its = [], [], []
    fast, _ = dp.gauss_newton_reconstruct(op, [0.0], w0=[0.01], n_iter=20,
                                          solver_mode="active_set", predict_only=predict,
                                          diagnostic_callback=events.append, update_log=log,
                                          iterates=its)
    np.testing.assert_allclose(fast, plain, rtol=1e-12, atol=1e-12)
    assert calls[0] < plain_calls and cheap[0] > 0
    assert events[-1]["projected_gradient"] <= 1e-6
    assert len(its) == 1 + sum(e["accepted"] for e in log)

    def cubic(w):
        return np.array([w[0] ** 3]), np.array([[3 * w[0] ** 2]])

    diagnostics = []
    rec, _ = dp.gauss_newton_reconstruct(cubic, [0.125], w0=[0.0001], n_iter=100,
                                         solver_mode="active_set", projected_gradient_tol=1e-12,
                                         diagnostics=diagnostics,
                                         predict_only=lambda w: np.array([w[0] ** 3]))
    np.testing.assert_allclose(rec, [0.5], atol=1e-8)
    assert diagnostics[-1]["projected_gradient"] < 1e-12
    assert np.all(np.diff([d["objective"] for d in diagnostics]) <= 0)

"""Inversion loops on the device (src/Tomography_inverse.jl consumers of the
forward model): one SART and one Gauss-Newton iteration against the same
update written out in numpy from the product's own Jacobian (FP64), and
convergence on a noise-free problem."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


@pytest.fixture(scope="module")
def problem(dp):
    import torch
    from dpgpu.workloads import density_field, detector_rays
    phys = dp.create_physics()
    nx, ny, nz, pitch = 16, 16, 8, 10.0
    origin = (-80.0, -80.0, 0.0)
    grid = dp.VoxelGrid(nx, ny, nz, origin, pitch)
    truth = density_field(nx, ny, nz, pitch, origin, seed=3, n_cavities=2,
                          radius=(15.0, 25.0)).ravel()
    rays = detector_rays([(-40.0, 0.0, 0.0), (40.0, 0.0, 0.0)], 96, 50.0, seed=4)
    nodes = dp.csda_energy_quadrature(16, 1.0, 1e6)
    paths = dp.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    dev = paths.dev
    T = lambda a: torch.tensor(np.ascontiguousarray(a, np.float64), device=dev)
    obs, _, _ = paths.eval(T(truth), precision="fp64")
    return dict(phys=phys, grid=grid, paths=paths, truth=truth, obs=obs, T=T, dev=dev)


def _jacobian(paths, rho_t):
    import torch
    jac = torch.empty(max(paths.nnz, 1), dtype=torch.float64, device=rho_t.device)
    f, _, _ = paths.eval(rho_t, precision="fp64", jac=jac)
    rp, col, _ = paths.csr()
    J = np.zeros((paths.n_rays, paths.grid.ncell))
    jv = jac.cpu().numpy()[:paths.nnz]
    for r in range(paths.n_rays):
        for p in range(rp[r], rp[r + 1]):
            if col[p] >= 0:
                J[r, col[p]] += jv[p]
    return f.cpu().numpy(), J


def test_sart_iteration_matches_numpy(dp, problem):
    """rho1 = clamp(rho0 + lambda D_col J^T D_row (obs - f(rho0)), box)."""
    paths, T = problem["paths"], problem["T"]
    n = paths.grid.ncell
    rho0 = np.full(n, 2650.0)
    box = (500.0, 3500.0)
    rho1, hist = paths.solve(problem["obs"], T(rho0), method="sart", n_iter=1, relaxation=0.2,
                             box=box, precision="fp64")
    f0, J = _jacobian(paths, T(rho0))
    obs = problem["obs"].cpu().numpy()
    r = obs - f0
    rows = np.abs(J).sum(1)
    rows[rows == 0] = 1.0
    cols = np.abs(J).sum(0)
    cols[cols == 0] = 1.0
    ref = np.clip(rho0 + 0.2 * (J.T @ (r / rows)) / cols, *box)
    np.testing.assert_allclose(rho1.cpu().numpy(), ref, rtol=1e-10, atol=1e-9)
    assert hist[0] == pytest.approx(np.linalg.norm(r), rel=1e-10)


def test_gauss_newton_iteration_matches_numpy(dp, problem):
    """One damped Gauss-Newton step: preconditioned CG on
    (J^T W J + mu max(D, 1e-12 max D)) d = -J^T W r, then the full step."""
    paths, T = problem["paths"], problem["T"]
    n = paths.grid.ncell
    rho0 = np.full(n, 2650.0)
    obs = problem["obs"].cpu().numpy()
    W = 1.0 / np.maximum(obs, 1e-30) ** 2 * 1e-4  # relative weights
    mu, K, box = 1e-3, 6, (500.0, 3500.0)
    rho1, hist = paths.solve(problem["obs"], T(rho0), method="gn", n_iter=1, weight=T(W),
                             cg_iter=K, lm_damping=mu, box=box, precision="fp64")
    f0, J = _jacobian(paths, T(rho0))
    r = f0 - obs
    g = J.T @ (W * r)
    D = (W[:, None] * J * J).sum(0)
    Df = np.maximum(D, 1e-12 * D.max())
    damp, prec = mu * Df, (1 + mu) * Df
    x = np.zeros(n)
    res = -g
    z = res / prec
    p = z.copy()
    rz = res @ z
    for _ in range(K):
        Ap = J.T @ (W * (J @ p)) + damp * p
        a = rz / (p @ Ap)
        x += a * p
        res -= a * Ap
        z = res / prec
        rz2 = res @ z
        p = z + rz2 / rz * p
        rz = rz2
    trial = np.clip(rho0 + x, *box)
    ft, _, _ = paths.eval(T(trial), precision="fp64")
    f_new = 0.5 * np.sum(W * (ft.cpu().numpy() - obs) ** 2)
    f_cur = 0.5 * np.sum(W * r ** 2)
    assert f_new < f_cur  # the full step is accepted
    np.testing.assert_allclose(rho1.cpu().numpy(), trial, rtol=1e-8, atol=1e-6)
    assert hist[0] == pytest.approx(np.linalg.norm(r), rel=1e-10)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gauss_newton_converges(dp, problem, precision):
    """Noise-free data: the misfit falls by a factor >= 10 and the density
    moves towards the truth."""
    paths, T = problem["paths"], problem["T"]
    n = paths.grid.ncell
    rho0 = np.full(n, 2650.0)
    obs = problem["obs"].cpu().numpy()
    W = 1.0 / np.maximum(obs, 1e-30) ** 2
    rho, hist = paths.solve(problem["obs"], T(rho0), method="gn", n_iter=6, weight=T(W),
                            precision=precision)
    done = hist[np.isfinite(hist)]
    assert done[-1] < 0.1 * done[0]
    assert np.all(np.diff(done) <= 1e-12 * done[0])
    truth = problem["truth"]
    seen = np.zeros(n, bool)
    rp, col, _ = paths.csr()
    seen[col[col >= 0]] = True
    rmse0 = np.sqrt(np.mean((rho0 - truth)[seen] ** 2))
    rmse = np.sqrt(np.mean((rho.cpu().numpy() - truth)[seen] ** 2))
    assert rmse < rmse0


def test_sart_reduces_misfit(dp, problem):
    paths, T = problem["paths"], problem["T"]
    rho0 = np.full(paths.grid.ncell, 2650.0)
    _, hist = paths.solve(problem["obs"], T(rho0), method="sart", n_iter=10, precision="mixed")
    assert hist[-1] < 0.8 * hist[0]


def test_smoothness_prior_gradient_step(dp, problem):
    """With the smoothness prior the Gauss-Newton objective adds
    weight * sum_edges (rho_i - rho_j)^2: a constant start has zero prior
    gradient, and the iterates stay smoother than without the prior."""
    paths, T = problem["paths"], problem["T"]
    g = paths.grid
    rho0 = np.full(g.ncell, 2650.0)
    obs = problem["obs"].cpu().numpy()
    W = 1.0 / np.maximum(obs, 1e-30) ** 2

    def roughness(x):
        x = x.reshape(g.nz, g.ny, g.nx)
        return sum(np.sum(np.diff(x, axis=a) ** 2) for a in range(3))

    free, _ = paths.solve(problem["obs"], T(rho0), method="gn", n_iter=4, weight=T(W),
                          precision="fp64")
    smooth, hist = paths.solve(problem["obs"], T(rho0), method="gn", n_iter=4, weight=T(W),
                               precision="fp64", prior_weight=1e-8)
    assert roughness(smooth.cpu().numpy()) < roughness(free.cpu().numpy())
    assert np.isfinite(hist[-1]) and hist[-1] < hist[0]


def test_gn_speculation_gives_the_same_iterates(dp, problem):
    """The speculative Jacobian (the first line-search trial evaluated with
    its Jacobian while first trials keep being accepted) changes which
    evaluations run, not the iterates.  A tiny initial damping makes early
    full steps overshoot, so the line search rejects trials, rebuilds the
    Jacobian at the iterate and later resumes speculating; the misfit history
    and the estimate equal those of a run that never speculates, bit for bit."""
    paths, T = problem["paths"], problem["T"]
    rho0 = T(np.full(paths.grid.ncell, 2650.0))
    runs = [paths.solve(problem["obs"], rho0, method="gn", n_iter=8, lm_damping=1e-9,
                        precision="mixed", speculation=s) for s in (True, False)]
    (r_on, h_on), (r_off, h_off) = runs
    np.testing.assert_array_equal(h_on, h_off)
    np.testing.assert_array_equal(r_on.cpu().numpy(), r_off.cpu().numpy())
    assert np.isfinite(h_on[0]) and np.nanmin(h_on[1:]) < h_on[0]


def _laplacian_dense(nx, ny, nz):
    n = nx * ny * nz
    L = np.zeros((n, n))
    idx = np.arange(n).reshape(nz, ny, nx)
    for a in range(3):
        lo, hi = [slice(None)] * 3, [slice(None)] * 3
        lo[a], hi[a] = slice(0, -1), slice(1, None)
        for i, j in zip(idx[tuple(lo)].ravel(), idx[tuple(hi)].ravel()):
            L[i, j] -= 1
            L[j, i] -= 1
            L[i, i] += 1
            L[j, j] += 1
    return L


@pytest.mark.parametrize("relinearize", [True, False])
def test_mlem_iterations_match_numpy(dp, problem, relinearize):
    """mlem_reconstruct (src/Tomography_inverse.jl:153-188) on the model
    linearised at the iterate (A = -J >= 0, b = max(f + A rho - obs, 0)), or
    once at the start: rho <- clamp(rho * A^T (b / max(A rho, 1e-12)) /
    (A^T 1 + max(2 lambda L rho, 0)), box), three iterations, FP64, against
    the same update in numpy on the product's Jacobian."""
    paths, T = problem["paths"], problem["T"]
    g = paths.grid
    n = g.ncell
    rho0 = np.full(n, 2650.0)
    obs = problem["obs"].cpu().numpy()
    prior, box = 1e-6, (500.0, 3500.0)
    rho_d, hist = paths.solve(problem["obs"], T(rho0), method="mlem", n_iter=3, box=box,
                              precision="fp64", prior_weight=prior, relinearize=relinearize)
    L = _laplacian_dense(g.nx, g.ny, g.nz)
    rho = np.maximum(rho0, 1e-6)
    f0, J0 = _jacobian(paths, T(rho))
    b0 = np.maximum(f0 - J0 @ rho - obs, 0.0)
    for it in range(3):
        f, J = (f0, J0) if (it == 0 or not relinearize) else _jacobian(paths, T(rho))
        if it > 0 and not relinearize:
            f = paths.eval(T(rho), precision="fp64")[0].cpu().numpy()
        assert hist[it] == pytest.approx(np.linalg.norm(obs - f), rel=1e-10)
        A = -J
        Aw = A @ rho
        b = b0 if not relinearize else np.maximum(f + Aw - obs, 0.0)
        sens = A.T @ np.ones(len(obs))
        sens[sens <= 0] = 1.0
        den = sens + np.maximum(2 * prior * (L @ rho), 0.0)
        rho = np.clip(rho * (A.T @ (b / np.maximum(Aw, 1e-12))) / den, *box)
    np.testing.assert_allclose(rho_d.cpu().numpy(), rho, rtol=1e-9, atol=1e-6)
    f_final = paths.eval(T(rho), precision="fp64")[0].cpu().numpy()
    assert hist[3] == pytest.approx(np.linalg.norm(obs - f_final), rel=1e-9)
    # the multiplicative step solves the linearised problem, not the flux
    # model, so it need not lower the flux misfit; only its bounds hold
    assert rho_d.min().item() >= box[0] and rho_d.max().item() <= box[1]


@pytest.mark.parametrize("optimizer,relinearize", [("pgd", True), ("pgd", False),
                                                   ("adam", True), ("gd", True)])
def test_gradient_descent_iterations_match_numpy(dp, problem, optimizer, relinearize):
    """gradient_descent_reconstruct (src/Tomography_inverse.jl:324-400) on
    0.5 sum W (f - obs)^2 + lambda sum_edges (rho_i - rho_j)^2: PGD (Jacobi
    preconditioner of the Gauss-Newton + prior diagonal, exact step capped at
    lr), Adam and plain steps, relinearised or with the start's linear model;
    four iterations, FP64, against the same loop in numpy."""
    paths, T = problem["paths"], problem["T"]
    g = paths.grid
    n = g.ncell
    rho0 = np.full(n, 2650.0)
    obs = problem["obs"].cpu().numpy()
    W = 1.0 / np.maximum(obs, 1e-30) ** 2
    prior, box = 1e-7, (500.0, 3500.0)
    lr = {"pgd": 1.0, "adam": 5.0, "gd": 1e-3}[optimizer]
    rho_d, hist = paths.solve(problem["obs"], T(rho0), method="gd", n_iter=4, weight=T(W),
                              box=box, precision="fp64", prior_weight=prior, optimizer=optimizer,
                              relinearize=relinearize, lr=lr)
    L = _laplacian_dense(g.nx, g.ny, g.nz)
    deg = np.diag(L)
    w = np.clip(rho0, *box)
    pred, J = _jacobian(paths, T(w))
    f0, J0, w0 = pred.copy(), J.copy(), w.copy()
    obj = lambda pr, x: 0.5 * np.sum(W * (pr - obs) ** 2) + prior * (x @ (L @ x))
    prev = obj(pred, w)
    m, v = np.zeros(n), np.zeros(n)
    ref_hist = [np.linalg.norm(pred - obs)]
    for t in range(1, 5):
        gr = J.T @ (W * (pred - obs)) + 2 * prior * (L @ w)
        if optimizer == "pgd":
            d = (W[:, None] * J * J).sum(0) + 2 * prior * deg
            dmax = d.max() if d.max() > 0 else 1.0
            p = gr / np.maximum(d, 1e-9 * dmax)
            Jp = J @ p
            denom = Jp @ (W * Jp) + p @ (2 * prior * (L @ p))
            num = gr @ p
            a = min(max(num / denom, 0.0), lr) if denom > 0 and np.isfinite(num) else 0.0
            w = np.clip(w - a * p, *box)
        elif optimizer == "adam":
            m = 0.9 * m + 0.1 * gr
            v = 0.999 * v + 0.001 * gr * gr
            w = np.clip(w - lr * (m / (1 - 0.9 ** t)) / (np.sqrt(v / (1 - 0.999 ** t)) + 1e-8),
                        *box)
        else:
            w = np.clip(w - lr * gr, *box)
        if relinearize:
            pred, J = _jacobian(paths, T(w))
        else:
            pred = f0 + J0 @ (w - w0)
        ref_hist.append(np.linalg.norm(pred - obs))
        o = obj(pred, w)
        if optimizer == "pgd" and abs(o - prev) <= 1e-5 * max(abs(prev), 2.2e-16):
            break
        prev = o
    np.testing.assert_allclose(rho_d.cpu().numpy(), w, rtol=1e-9, atol=1e-6)
    k = len(ref_hist)
    np.testing.assert_allclose(hist[:k], ref_hist, rtol=1e-9)
    assert np.isnan(hist[k:]).all()
    if optimizer == "pgd" and relinearize:
        f_final = paths.eval(T(w), precision="fp64")[0].cpu().numpy()
        assert np.linalg.norm(obs - f_final) < ref_hist[0]

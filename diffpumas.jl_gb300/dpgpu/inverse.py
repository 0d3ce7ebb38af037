"""Inverse solvers of src/Tomography_inverse.jl over the device operator.

The unknown is the per-cell water fraction w in [0, MAX_WATER_FRACTION].  The
solvers are the reference's algorithms (SART, MLEM, projected gradient /
Adam, damped Gauss-Newton) on a sparse Jacobian; `make_csda_operator`
returns the model(w) -> (pred, J) closure whose flux and Jacobian come from
the water-fraction CSDA kernel (one launch for all bins).  The voxel-density
loops that keep everything on the device are TomoPaths.solve.
"""
import math

import numpy as np

MAX_WATER_FRACTION = 0.9  # src/Tomography.jl:88


def _sparse():
    import scipy.sparse as sp
    return sp


# ------------------------------------------------------------------ priors
def _undirected(neighbors):
    """Unique undirected, sorted adjacency without self loops (:25-34)."""
    n = len(neighbors)
    graph = [set() for _ in range(n)]
    for i, nb in enumerate(neighbors):
        for j in nb:
            j = int(j)
            if not 0 <= j < n:
                raise ValueError(f"Prior neighbor index {j} is outside 0:{n - 1}")
            if i != j:
                graph[i].add(j)
                graph[j].add(i)
    return [sorted(g) for g in graph]


class SmoothnessPrior:
    """R(w) = weight * sum over unique edges (w_i - w_j)^2 (:36-41).
    Cells are 0-based here."""

    def __init__(self, neighbors, weight):
        self.neighbors = _undirected(neighbors)
        self.weight = float(weight)


class EdgePrior:
    """Huber edge-preserving prior weight * sum rho_delta(w_i - w_j) (:205-211)."""

    def __init__(self, neighbors, weight, delta):
        self.neighbors = _undirected(neighbors)
        self.weight = float(weight)
        self.delta = float(delta)


def _edges(prior):
    return [(i, j) for i, nb in enumerate(prior.neighbors) for j in nb if i < j]


def laplacian_gradient(prior, w):
    """dR/dw = 2 weight sum_{j in N(k)} (w_k - w_j) (:43-61)."""
    w = np.asarray(w, np.float64)
    g = np.zeros(len(w))
    for k, nb in enumerate(prior.neighbors):
        g[k] = 2.0 * prior.weight * sum(w[k] - w[j] for j in nb)
    return g


def apply_laplacian_smoothing(prior, w, strength):
    """One sweep w_k <- (1 - s) w_k + s mean(w_neighbours) (:63-80)."""
    w = np.asarray(w, np.float64)
    out = w.copy()
    for k, nb in enumerate(prior.neighbors):
        if nb:
            out[k] = (1.0 - strength) * w[k] + strength * float(np.mean(w[nb]))
    return out


def _huber_grad(t, d):
    return t if abs(t) <= d else d * math.copysign(1.0, t)


def _huber_irls(t, d):
    return 1.0 if abs(t) <= d else d / abs(t)


def edge_gradient(prior, w):
    """dR/dw of the Huber prior (:216-229)."""
    w = np.asarray(w, np.float64)
    g = np.zeros(len(w))
    for k, nb in enumerate(prior.neighbors):
        g[k] = prior.weight * sum(_huber_grad(w[k] - w[j], prior.delta) for j in nb)
    return g


def edge_hessian(prior, w):
    """Lagged-diffusivity Hessian weight * L^psi (:231-249), sparse."""
    sp = _sparse()
    w = np.asarray(w, np.float64)
    rows, cols, vals = [], [], []
    for k, nb in enumerate(prior.neighbors):
        diag = 0.0
        for j in nb:
            psi = _huber_irls(w[k] - w[j], prior.delta)
            diag += psi
            rows.append(k)
            cols.append(j)
            vals.append(-prior.weight * psi)
        rows.append(k)
        cols.append(k)
        vals.append(prior.weight * diag)
    n = len(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def prior_value(prior, w):
    """The prior's objective (:251-273)."""
    if prior is None:
        return 0.0
    w = np.asarray(w, np.float64)
    total = 0.0
    if isinstance(prior, EdgePrior):
        d = prior.delta
        for i, j in _edges(prior):
            a = abs(w[i] - w[j])
            total += 0.5 * a * a if a <= d else d * (a - 0.5 * d)
    else:
        for i, j in _edges(prior):
            total += (w[i] - w[j]) ** 2
    return prior.weight * total


def _prior_grad(prior, w):
    return edge_gradient(prior, w) if isinstance(prior, EdgePrior) else laplacian_gradient(prior, w)


def _prior_hessian(prior, w):
    """The Gauss-Newton curvature of the prior (:274-275): the smoothness
    prior is the Huber one with twice the weight and delta = inf."""
    if isinstance(prior, EdgePrior):
        return edge_hessian(prior, w)
    return edge_hessian(EdgePrior(prior.neighbors, 2.0 * prior.weight, math.inf), w)


# ------------------------------------------------------------------ linear solvers
def sart_reconstruct(A, b, *, w0=None, n_iter=50, relaxation=0.2, box=(0.0, MAX_WATER_FRACTION),
                     prior=None, smooth_strength=0.1, free=None, snapshots=None,
                     snapshot_iters=()):
    """SART on A w ~ b (:98-132): w <- clamp(w + relaxation D_col A^T D_row
    (b - A w), box), an optional smoothing sweep, free-mask cells fixed at 0."""
    sp = _sparse()
    A = sp.csr_matrix(A)
    n = A.shape[1]
    w = np.zeros(n) if w0 is None else np.array(w0, np.float64)
    b = np.asarray(b, np.float64)
    if free is not None:
        free = np.asarray(free, bool)
        if len(free) != n:
            raise ValueError("free mask must match the columns of A")
        A = A @ sp.diags(free.astype(np.float64))
        w[~free] = 0.0
    Aabs = abs(A)
    rows = np.asarray(Aabs.sum(axis=1)).ravel()
    cols = np.asarray(Aabs.sum(axis=0)).ravel()
    rows[rows == 0] = 1.0
    cols[cols == 0] = 1.0
    history = []
    for _ in range(n_iter):
        r = b - A @ w
        w = np.clip(w + relaxation * (A.T @ (r / rows)) / cols, *box)
        if prior is not None:
            w = np.clip(apply_laplacian_smoothing(prior, w, smooth_strength), *box)
        if free is not None:
            w[~free] = 0.0
        history.append(float(np.linalg.norm(b - A @ w)))
        if snapshots is not None and len(history) in snapshot_iters:
            snapshots[len(history)] = w.copy()
    return w, history


def mlem_reconstruct(A, b, *, w0=None, n_iter=100, box=(0.0, MAX_WATER_FRACTION), prior=None,
                     eps=1e-12, free=None, snapshots=None, snapshot_iters=()):
    """Multiplicative EM for A >= 0, b >= 0 (:153-188): w <- w (A^T (b / Aw)) /
    (A^T 1 + max(dR/dw, 0)), clamped to the box; one-step-late prior."""
    sp = _sparse()
    A = sp.csr_matrix(A)
    n = A.shape[1]
    w = np.full(n, max(box[0], 1e-3)) if w0 is None else np.array(w0, np.float64)
    w = np.maximum(w, 1e-6)  # a multiplicative update cannot leave 0
    b = np.asarray(b, np.float64)
    if free is not None:
        free = np.asarray(free, bool)
        if len(free) != n:
            raise ValueError("free mask must match the columns of A")
        A = A @ sp.diags(free.astype(np.float64))
        w[~free] = 0.0
    sens = np.asarray(A.sum(axis=0)).ravel()
    sens[sens <= 0] = 1.0
    history = []
    for _ in range(n_iter):
        Aw = np.maximum(A @ w, eps)
        ratio = A.T @ (b / Aw)
        denom = sens.copy()
        if prior is not None:
            denom = denom + np.maximum(laplacian_gradient(prior, w), 0.0)
        w = np.clip(w * ratio / denom, *box)
        if free is not None:
            w[~free] = 0.0
        history.append(float(np.linalg.norm(b - A @ w)))
        if snapshots is not None and len(history) in snapshot_iters:
            snapshots[len(history)] = w.copy()
    return w, history


# ------------------------------------------------------------------ nonlinear solvers
def gradient_descent_reconstruct(model, obs, *, w0, n_iter=200, lr=1e-2,
                                 box=(0.0, MAX_WATER_FRACTION), prior=None, optimizer="adam",
                                 relinearize=True, weights=None, free=None, snapshots=None):
    """Projected gradient descent on 1/2 |pred(w) - obs|^2_W + R(w) (:277-400).
    optimizer: "pgd" (Jacobi-preconditioned, exact step on the local
    quadratic model, capped at lr), "adam" or "gd"."""
    w = np.clip(np.array(w0, np.float64), *box)
    obs = np.asarray(obs, np.float64)
    if free is not None:
        free = np.asarray(free, bool)
        if len(free) != len(w):
            raise ValueError("free mask must match w0")
        if optimizer != "pgd":
            raise ValueError("free requires optimizer='pgd'")
    history = []
    if n_iter <= 0:
        return w, history
    W = None if weights is None else np.asarray(weights, np.float64)

    def data_cost(r):
        return 0.5 * float(r @ r) if W is None else 0.5 * float(np.sum(W * r * r))

    m = np.zeros(len(w))
    v = np.zeros(len(w))
    b1, b2, e = 0.9, 0.999, 1e-8
    pred, J = model(w)
    origin, pred0, J0 = w.copy(), np.array(pred), J
    previous = data_cost(pred - obs) + prior_value(prior, w)
    for t in range(1, n_iter + 1):
        r = pred - obs
        g = J.T @ (r if W is None else W * r)
        if prior is not None:
            g = g + _prior_grad(prior, w)
        if optimizer == "pgd":
            J2 = J.multiply(J)
            dvec = np.asarray((J2 if W is None else J2.multiply(W[:, None])).sum(axis=0)).ravel()
            Hr = None if prior is None else _prior_hessian(prior, w)
            if Hr is not None:
                dvec = dvec + Hr.diagonal()
            dmax = dvec.max() if dvec.size and dvec.max() > 0 else 1.0
            p = g / np.maximum(dvec, 1e-9 * dmax)
            if free is not None:
                p[~free] = 0.0
            Jp = J @ p
            denom = float(Jp @ Jp) if W is None else float(Jp @ (W * Jp))
            if Hr is not None:
                denom += float(p @ (Hr @ p))
            num = float(g @ p)
            alpha = min(max(num / denom, 0.0), lr) if denom > 0 and math.isfinite(num) else 0.0
            w = np.clip(w - alpha * p, *box)
        elif optimizer == "adam":
            m = b1 * m + (1 - b1) * g
            v = b2 * v + (1 - b2) * g * g
            w = np.clip(w - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + e), *box)
        else:
            w = np.clip(w - lr * g, *box)
        if relinearize:
            pred, J = model(w)
        else:
            pred, J = pred0 + J0 @ (w - origin), J0
        objective = data_cost(pred - obs) + prior_value(prior, w)
        history.append(float(np.linalg.norm(pred - obs)))
        if snapshots is not None:
            snapshots[t] = w.copy()
        if optimizer == "pgd" and abs(objective - previous) <= 1e-5 * max(abs(previous), 2.2e-16):
            break
        previous = objective
    return w, history


def _gn_accept_trial(f_new, f_cur, grad, step, mode):
    """Acceptance of a trial point (src/Tomography_inverse.jl:441-446):
    legacy needs a relative decrease of 1e-10; active_set needs a descent
    direction and the Armijo condition with c = 1e-4."""
    if not math.isfinite(f_new):
        return False
    if mode == "legacy":
        return f_new < f_cur - 1e-10 * abs(f_cur)
    directional = float(np.dot(grad, step))
    return directional < 0 and f_new < f_cur and f_new <= f_cur + 1e-4 * directional


def _normal_equations(J, active, W, r, prior, w):
    Ja = J[:, active]
    if _issparse(Ja):
        if W is None:
            normal, grad = (Ja.T @ Ja).toarray(), Ja.T @ r
        else:
            normal, grad = (Ja.T @ Ja.multiply(W[:, None]).tocsr()).toarray(), Ja.T @ (W * r)
    else:
        Ja = np.asarray(Ja, np.float64)
        if W is None:
            normal, grad = Ja.T @ Ja, Ja.T @ r
        else:
            normal, grad = Ja.T @ (W[:, None] * Ja), Ja.T @ (W * r)
    grad = np.asarray(grad, np.float64).ravel()
    if prior is not None:
        grad = grad + _prior_grad(prior, w)[active]
        normal = normal + _prior_hessian(prior, w)[active][:, active].toarray()
    return normal, grad


def _issparse(x):
    return _sparse().issparse(x)


def gauss_newton_reconstruct(model, obs, *, w0, n_iter=12, box=(0.0, MAX_WATER_FRACTION),
                             prior=None, lm_damping=1e-3, lm_factor=3.0, relinearize=True,
                             weights=None, free=None, predict_only=None, solver_mode="legacy",
                             projected_gradient_tol=1e-6, objective_tol=0.0, diagnostics=None,
                             diagnostic_callback=None, rel_objective_tol=0.0, iterates=None,
                             update_log=None, stop=None):
    """Box-constrained Levenberg-Marquardt on the regularised normal equations
    (J^T W J + H_R + mu diag) delta = -(J^T W r + grad R) (src/Tomography_inverse.jl:448-603).

    solver_mode "legacy": 6 damping levels x 14 halvings, accepting a
    relative decrease of 1e-10.  "active_set": coordinates at a bound whose
    gradient points outward are frozen, a projected Newton direction that is
    not descent falls back to the diagonally scaled gradient, acceptance is
    projected Armijo, a seventh try takes a bounded scaled-gradient step with
    up to 40 halvings, and the loop stops once the infinity norm of the
    projected gradient is at most projected_gradient_tol.  predict_only(w)
    gives the prediction for line-search trials; an accepted trial is checked
    again with the full model.  diagnostics (a list) and diagnostic_callback
    receive {iteration, objective, projected_gradient} records, the final
    state included; iterates receives w0 and every accepted iterate;
    update_log one record per update; stop (a one-element list) the stop
    reason: max_updates, projected_gradient, no_step, objective_decrease or
    no_free_cells."""
    if solver_mode not in ("legacy", "active_set"):
        raise ValueError("unknown solver_mode")
    legacy = solver_mode == "legacy"
    lo, hi = box
    w = np.clip(np.array(w0, np.float64), lo, hi)
    obs = np.asarray(obs, np.float64)
    if free is not None and len(free) != len(w):
        raise ValueError("free mask must match w0")
    active = np.arange(len(w)) if free is None else np.nonzero(np.asarray(free, bool))[0]
    W = None if weights is None else np.asarray(weights, np.float64)

    def record(row):
        if diagnostics is not None:
            diagnostics.append(row)
        if diagnostic_callback is not None:
            diagnostic_callback(row)

    def objective(pred, wv):
        r = np.asarray(pred, np.float64) - obs
        data = 0.5 * float(r @ r) if W is None else 0.5 * float(np.sum(W * r * r))
        return data + prior_value(prior, wv)

    pred, J = model(w)
    pred = np.asarray(pred, np.float64)
    origin, pred0, J0 = w.copy(), pred.copy(), J
    r = pred - obs
    f_cur = objective(pred, w)
    mu = lm_damping
    history = [float(np.linalg.norm(r))]
    if iterates is not None:
        iterates.append(w.copy())
    if stop is not None:
        stop[:] = ["max_updates"]
    if len(active) == 0:
        if stop is not None:
            stop[:] = ["no_free_cells"]
        return w, history
    for update in range(1, n_iter + 1):
        normal, grad = _normal_equations(J, active, W, r, prior, w)
        wa = w[active]
        pg_norm = float(np.max(np.abs(wa - np.clip(wa - grad, lo, hi))))
        record({"iteration": len(history) - 1, "objective": f_cur, "projected_gradient": pg_norm})
        if not legacy and pg_norm <= projected_gradient_tol:
            if stop is not None:
                stop[:] = ["projected_gradient"]
            break
        movable = (np.ones(len(active), bool) if legacy else
                   ~(((wa <= lo) & (grad > 0)) | ((wa >= hi) & (grad < 0))))
        d = np.diag(normal).copy()
        dmax = d.max() if d.max() > 0 else 1.0
        accepted = False
        f_before, mu_before, tries = f_cur, mu, 0
        for attempt in range(1, (6 if legacy else 7) + 1):
            tries += 1
            A = normal + np.diag(mu * np.maximum(d, 1e-12 * dmax))
            rescue = not legacy and attempt == 7
            if rescue:
                delta = -grad / np.maximum(np.maximum(d, np.max(np.abs(grad))), 1e-30)
            else:
                try:
                    delta = np.zeros(len(active))
                    m = np.nonzero(movable)[0]
                    delta[m] = -np.linalg.solve(A[np.ix_(m, m)], grad[m])
                    if not legacy:
                        projected = np.clip(wa + delta, lo, hi) - wa
                        if float(grad @ projected) >= 0:
                            delta = -grad / np.maximum(d, 1e-12 * dmax)
                except np.linalg.LinAlgError:
                    delta = (np.zeros(len(active)) if legacy else
                             -grad / np.maximum(d, 1e-12 * dmax))
            if not np.all(np.isfinite(delta)):
                mu = min(mu * lm_factor, 1e12)
                continue
            alpha = 1.0
            cached = None
            for _ls in range(40 if rescue else 14):
                w_new = w.copy()
                w_new[active] = np.clip(wa + alpha * delta, lo, hi)
                if np.array_equal(w_new, w):
                    break
                if cached is not None and np.array_equal(w_new, cached[0]):
                    pred_new, J_new = cached[1], cached[2]
                elif relinearize and predict_only is not None:
                    pred_new, J_new = np.asarray(predict_only(w_new), np.float64), None
                    cached = (w_new, pred_new, None)
                else:
                    if relinearize:
                        pred_new, J_new = model(w_new)
                    else:
                        pred_new, J_new = pred0 + J0 @ (w_new - origin), J0
                    pred_new = np.asarray(pred_new, np.float64)
                    cached = (w_new, pred_new, J_new)
                f_new = objective(pred_new, w_new)
                step = w_new[active] - wa
                if _gn_accept_trial(f_new, f_cur, grad, step, solver_mode):
                    if relinearize and predict_only is not None and J_new is None:
                        pred_new, J_new = model(w_new)
                        pred_new = np.asarray(pred_new, np.float64)
                        f_new = objective(pred_new, w_new)
                        cached = (w_new, pred_new, J_new)
                    if _gn_accept_trial(f_new, f_cur, grad, step, solver_mode):
                        w, r, J, pred, f_cur = w_new, pred_new - obs, J_new, pred_new, f_new
                        accepted = True
                        break
                alpha *= 0.5
            if accepted:
                mu = max(mu / lm_factor, 1e-12)
                break
            mu = min(mu * lm_factor, 1e12)
        history.append(float(np.linalg.norm(r)))
        if update_log is not None:
            update_log.append({"update": update, "objective_before": f_before,
                               "objective_after": f_cur, "projected_gradient": pg_norm,
                               "damping": mu_before, "tries": tries, "accepted": accepted})
        if not accepted:
            if stop is not None:
                stop[:] = ["no_step"]
            break
        if iterates is not None:
            iterates.append(w.copy())
        if rel_objective_tol > 0 and f_before - f_cur < rel_objective_tol * abs(f_before):
            if stop is not None:
                stop[:] = ["objective_decrease"]
            break
        if (not legacy and objective_tol > 0 and
                abs(f_before - f_cur) <= objective_tol * max(1.0, abs(f_before))):
            break
    if diagnostics is not None or diagnostic_callback is not None:
        _, grad = _normal_equations(J, active, W, r, prior, w)
        wa = w[active]
        record({"iteration": len(history) - 1, "objective": f_cur,
                "projected_gradient": float(np.max(np.abs(wa - np.clip(wa - grad, lo, hi))))})
    return w, history


# ------------------------------------------------------------------ operator and metrics
def make_csda_operator(physics, shallow_flags, matcfg, site, paths, energy_samples, *, n_cells,
                       valid_bins, threaded=True, precision="fp64"):
    """model(w) -> (pred, J) over the bins valid_bins (0-based) (:614-626):
    the water-fraction CSDA flux and its sparse Jacobian from one device
    launch over all bins."""
    from .directional import CsdaBatch
    import scipy.sparse as sp
    sub = [paths[i] for i in valid_bins]
    batch = CsdaBatch(physics, shallow_flags, matcfg, site, sub, energy_samples)
    rows = np.repeat(np.arange(len(sub)), np.diff(batch.arrays["seg_ptr"]))
    cols = batch.arrays["seg_cell"]

    def model(w):
        flux, jac = batch.run(w, precision=precision)
        J = sp.csr_matrix((jac, (rows, cols)), shape=(len(sub), n_cells))
        J.sum_duplicates()
        J.data[~np.isfinite(J.data)] = 0.0
        J.eliminate_zeros()
        return flux, J

    return model


def mse(recon, truth, mask=None):
    a = np.asarray(recon, np.float64)
    b = np.asarray(truth, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    return float(np.mean((a - b) ** 2))


def rmse(recon, truth, mask=None):
    """src/Tomography_inverse.jl:642."""
    return math.sqrt(mse(recon, truth, mask))

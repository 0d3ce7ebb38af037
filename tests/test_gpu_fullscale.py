"""Parity at the benchmarked sizes of the configurations (C2, C4, C5), through
the C ABI, against the FP64 oracle on the same inputs.

- C2: the straggled + scattering transport of 10^6 histories through the
  rock/water/air mixture (the bench's workload, mixed precision) against the
  oracle on the first 10^5 histories of the same Philox streams, and the
  mixed-precision histories of those 10^5 paired one by one with the oracle's.
- C4: all 16,384 lines of sight of the bench's generator (8.9 million
  histories, uneven depths and sample counts) in one mixed-precision batch;
  64 seeded lines of sight against the oracle's histories and CSDA gradients,
  and their FP64 histories (same stream ids) one by one against the oracle.
- C5: one Gauss-Newton iteration on the 128 x 128 x 64 grid with 8 x 8192 rays
  (FP64, smoothness prior) against the same update written out with
  scipy.sparse from the product's own Jacobian, and a five-iteration
  Gauss-Newton loop on a 32 x 32 x 16 grid against the same loop driven by the
  oracle's forward model and Jacobian.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


@pytest.fixture(scope="module")
def orc3(oracle):
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), coulomb=True)


@pytest.fixture(scope="module")
def phys3(dp, orc3):
    tabs = [orc3.table(i) for i in range(3)]
    return dp.upload_physics(tabs, ["StandardRock", "Air", "Water"],
                             materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))


def _flux_sigma(c):
    f = c.mean()
    return f, math.sqrt(max((c * c).mean() - f * f, 0.0) / len(c))


# ------------------------------------------------------------------ C2
def test_c2_full_scale_against_oracle(dp, phys3, oracle, orc3):
    """10^6 mixed-precision histories (per-history thickness U[20,500] m,
    density U[2000,2800], elevation U[30,90] deg drawn on the device, 1 km of
    air above, E log-uniform 1 GeV - 10 TeV): the batch flux lies within 3
    sigma of the oracle's FP64 flux over the first 10^5 histories of the same
    streams (the oracle's sigma dominates), and on those 10^5 histories the
    mixed-minus-FP64 paired differences average to zero within 3 of their
    standard errors."""
    seed, n, m = 2026, 1_000_000, 100_000
    mix = dp.MaterialMixture(phys3, [1, 3, 2], [0.70, 0.25, 0.05])
    air = dp.MaterialMixture(phys3, 2)
    rng = dict(thickness=20.0, thickness_max=500.0, density=2000.0, density_max=2800.0,
               elevation=30.0, elevation_max=90.0)
    los = dp.make_los(n, air_height=1000.0, energy_min=1.0, energy_max=1e4, **rng)
    r = dp.backward_mc_batch(phys3, los, rock=mix, air=air, seed=seed, precision="mixed")
    assert r["n_status_nonzero"][0] == 0 and r["n_samples"][0] == n
    ids = np.arange(m)
    E, q, w = oracle.energy_draws(seed, ids, 1.0, 1e4)
    t, rho, el = oracle.los_geometry_draws(seed, ids, **rng)
    oc, ost, _, _ = oracle.mc_histories(orc3, [0, 2, 1], 1, t, rho, el, t + 1000.0, E, q, w,
                                        seed=seed, rock_fracs=[0.70, 0.25, 0.05])
    assert (ost == 0).all()
    fo, so = _flux_sigma(oc)
    z = (r["flux"][0] - fo) / math.hypot(r["sigma"][0], so)
    assert abs(z) < 3, (r["flux"][0], fo, so)
    # the same 10^5 histories, mixed precision, one by one
    mc, mst, _, _ = dp.mc_histories(phys3, mix, air, E, q, w, thickness=t, density=rho,
                                    elevation=el, primary_altitude=t + 1000.0, seed=seed,
                                    precision="mixed")
    assert (mst == 0).all()
    d = mc - oc
    zd = d.mean() / (d.std() / math.sqrt(m))
    assert abs(zd) < 3, (d.mean(), d.std())
    # a large share of the histories end alike (47 % on this workload: with
    # scattering on, a sampling decision flipped by FP32 rounding sends a
    # history elsewhere; that is the statistical part checked above)
    same = np.abs(mc - oc) <= 1e-3 * np.maximum(np.abs(mc), np.abs(oc)) + 1e-300
    assert same.mean() > 0.35


# ------------------------------------------------------------------ C4
def _c4_los(dp, seed=4, n_los=16384):
    rng = np.random.default_rng(seed)
    depth = np.exp(rng.uniform(np.log(50.0), np.log(2000.0), n_los))
    rho = rng.uniform(2400.0, 2800.0, n_los)
    ns = rng.integers(64, 1025, n_los)
    return dp.make_los(ns, thickness=depth, density=rho, elevation=90.0, energy_min=1.0,
                       energy_max=1e4), depth, rho, ns


@pytest.fixture(scope="module")
def orc2(oracle):
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR), coulomb=True)


@pytest.fixture(scope="module")
def c4_runs(dp, orc2):
    """The full C4 batch in mixed precision (one launch per phase), and the
    64 seeded lines' histories."""
    phys = dp.upload_physics([orc2.table(0), orc2.table(1)], ["StandardRock", "Air"],
                             materials=(dp.STANDARD_ROCK, dp.AIR))
    rock, air = dp.MaterialMixture(phys, 1), dp.MaterialMixture(phys, 2)
    los, depth, rho, ns = _c4_los(dp)
    mixed = dp.backward_mc_batch(phys, los, rock=rock, air=air, seed=2027, scattering=False,
                                 energy_threshold_low=1.0, compute_gradient=True,
                                 precision="mixed")
    pick = np.sort(np.random.default_rng(64).choice(len(ns), 64, replace=False))
    return phys, rock, air, depth, rho, ns, mixed, pick


def test_c4_full_scale_lines_against_oracle(dp, oracle, orc2, c4_runs):
    """All 16,384 lines of sight (8.9 million histories, depths 50-2000 m,
    64-1024 histories each) in one mixed-precision batch; 64 seeded lines
    against the FP64 oracle on the same histories (history id = running
    sample index): every line's mixed flux within 3 sigma of the oracle's
    (the two transports follow the same draws, so the RMS z is far below 1),
    and the CSDA sample-average flux and d flux/d rho within 1e-6 of the
    oracle's dual numbers (the FP32 CSDA walk)."""
    phys, rock, air, depth, rho, ns, mixed, pick = c4_runs
    assert (mixed["n_status_nonzero"] == 0).all() and (mixed["n_samples"] == ns).all()
    assert np.isfinite(mixed["flux"]).all() and (mixed["flux"] >= 0).all()
    off = np.concatenate([[0], np.cumsum(ns)])
    zs = []
    for l in pick:
        ids = np.arange(off[l], off[l + 1])
        E, q, w = oracle.energy_draws(2027, ids, 1.0, 1e4)
        oc, ost, _, _ = oracle.mc_histories(orc2, [0], 1, depth[l], rho[l], 90.0, 3e4, E, q, w,
                                            seed=2027, id0=int(off[l]), straggling=True,
                                            scattering=False, threshold_low=1.0)
        assert (ost == 0).all()
        fo, so = _flux_sigma(oc)
        zs.append((mixed["flux"][l] - fo) / so)
        cc, cd = oracle.backward_mc_csda(orc2, 0, 1, depth[l], rho[l], 90.0, E, q, w)
        assert mixed["gradient_flux"][l] == pytest.approx(cc.mean(), rel=1e-6,
                                                          abs=1e-12 * abs(cc).max())
        assert mixed["gradient"][l] == pytest.approx(cd.mean(), rel=1e-6,
                                                     abs=1e-12 * abs(cd).max())
    zs = np.array(zs)
    assert np.abs(zs).max() < 3, zs
    assert np.sqrt(np.mean(zs ** 2)) < 0.5, zs


def test_c4_fp64_histories_of_the_full_scale_lines(dp, oracle, orc2, c4_runs):
    """The FP64 transport of the same 64 lines' histories (explicit
    histories with the batch's stream ids; the FP64 form of all 8.9 million
    histories would take minutes at GB300's FP64 rate): at least 95 % of the
    histories equal the oracle's to 1e-9 (a sampling decision flipped by the
    last bit of a transcendental is the rest), the line flux within half a
    sigma, and the batch's mixed flux of each line within 3 sigma of it."""
    phys, rock, air, depth, rho, ns, mixed, pick = c4_runs
    off = np.concatenate([[0], np.cumsum(ns)])
    agree, total = 0, 0
    for l in pick:
        ids = np.arange(off[l], off[l + 1])
        E, q, w = oracle.energy_draws(2027, ids, 1.0, 1e4)
        oc, _, _, _ = oracle.mc_histories(orc2, [0], 1, depth[l], rho[l], 90.0, 3e4, E, q, w,
                                          seed=2027, id0=int(off[l]), straggling=True,
                                          scattering=False, threshold_low=1.0)
        c, st, _, _ = dp.mc_histories(phys, rock, air, E, q, w, thickness=depth[l],
                                      density=rho[l], elevation=90.0, primary_altitude=3e4,
                                      seed=2027, id0=int(off[l]), scattering=False,
                                      energy_threshold_low=1.0, precision="fp64")
        assert (st == 0).all()
        same = np.abs(c - oc) <= 1e-9 * np.maximum(np.abs(c), np.abs(oc)) + 1e-300
        agree += same.sum()
        total += len(c)
        f, s = _flux_sigma(c)
        fo, so = _flux_sigma(oc)
        assert abs(f - fo) <= max(0.5 * so, 1e-9 * abs(fo)), (l, f, fo, so)
        assert abs(mixed["flux"][l] - f) < 3 * s, (l, mixed["flux"][l], f, s)
    assert agree >= 0.95 * total, agree / total


# ------------------------------------------------------------------ C5
def _laplacian(nx, ny, nz):
    """Graph Laplacian of the grid's 6-neighbour edges (x fastest)."""
    import scipy.sparse as sp
    idx = np.arange(nx * ny * nz).reshape(nz, ny, nx)
    rows, cols = [], []
    for a in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[a], hi[a] = slice(0, -1), slice(1, None)
        rows.append(idx[tuple(lo)].ravel())
        cols.append(idx[tuple(hi)].ravel())
    i, j = np.concatenate(rows), np.concatenate(cols)
    n = nx * ny * nz
    A = sp.coo_matrix((np.ones(i.size), (i, j)), shape=(n, n))
    A = (A + A.T).tocsr()
    return (sp.diags(np.asarray(A.sum(1)).ravel()) - A).tocsr()


def _gn_restated(J_of, f_of, obs, W, rho0, L, prior, n_iter, cg_iter=10, mu=1e-3,
                 box=(500.0, 3500.0)):
    """The device's Gauss-Newton loop written out with scipy.sparse: damped
    normal equations (J^T W J + mu max(D, 1e-12 max D) + 2 prior L) d =
    -(J^T W r + 2 prior L rho) by Jacobi-preconditioned CG from 0, then the
    legacy backtracking line search (accept f_new < f - 1e-10 |f|; 6 damping
    attempts x 14 halvings; mu / 3 on acceptance, x 3 otherwise).  Returns
    the iterate and the misfit history ||f(rho) - obs||."""
    rho = rho0.copy()
    # sum over edges of (x_i - x_j)^2 equals x^T L x
    objective = lambda f, x: 0.5 * np.sum(W * (f - obs) ** 2) + prior * (x @ (L @ x))
    f = f_of(rho)
    f_cur = objective(f, rho)
    hist = []
    deg = L.diagonal()
    for _ in range(n_iter):
        hist.append(np.linalg.norm(f - obs))
        J = J_of(rho)
        r = f - obs
        g = J.T @ (W * r) + 2 * prior * (L @ rho)
        D = J.multiply(J).T @ W + 2 * prior * deg
        dmax = D.max() if D.max() > 0 else 1.0
        accepted = False
        for _attempt in range(6):
            Df = np.maximum(D, 1e-12 * dmax)
            damp, prec = mu * Df, (1 + mu) * Df
            x = np.zeros_like(rho)
            res = -g
            z = res / prec
            p = z.copy()
            rz = res @ z
            for _k in range(cg_iter):
                Ap = J.T @ (W * (J @ p)) + damp * p + 2 * prior * (L @ p)
                a = rz / (p @ Ap)
                x += a * p
                res -= a * Ap
                z = res / prec
                rz2 = res @ z
                p = z + rz2 / rz * p
                rz = rz2
            alpha = 1.0
            for _ls in range(14):
                trial = np.clip(rho + alpha * x, *box)
                ft = f_of(trial)
                fn = objective(ft, trial)
                if np.isfinite(fn) and fn < f_cur - 1e-10 * abs(f_cur):
                    rho, f, f_cur, accepted = trial, ft, fn, True
                    break
                alpha *= 0.5
            mu = max(mu / 3, 1e-12) if accepted else min(mu * 3, 1e12)
            if accepted:
                break
        if not accepted:
            break
    hist.append(np.linalg.norm(f - obs))
    return rho, np.array(hist)


def _device_jacobian(paths, rho_t):
    import scipy.sparse as sp
    import torch
    jac = torch.empty(max(paths.nnz, 1), dtype=torch.float64, device=rho_t.device)
    f, _, _ = paths.eval(rho_t, precision="fp64", jac=jac)
    rp, col, _ = paths.csr()
    jv = jac.cpu().numpy()[:paths.nnz]
    keep = col >= 0  # side-exit remainders sit at a fixed density
    rows = np.repeat(np.arange(paths.n_rays), np.diff(rp))
    J = sp.csr_matrix((jv[keep], (rows[keep], col[keep])), shape=(paths.n_rays, paths.grid.ncell))
    J.sum_duplicates()
    return f.cpu().numpy(), J


def test_c5_full_scale_gauss_newton_iteration(dp):
    """The bench's C5 problem (128 x 128 x 64 at 10 m, 8 x 8192 rays, Poisson
    counts ~10^3 per ray, W = tau^2 / max(counts, 1), prior 1e-5, start 2650):
    one device Gauss-Newton iteration in FP64 equals the scipy restatement on
    the product's Jacobian (an independently pinned quantity: segments equal
    the oracle's, flux and gradients within 1e-9 / 1e-6 of it)."""
    import torch
    from dpgpu.workloads import tomography_config
    grid, truth, rays, nodes = tomography_config(nx=128, ny=128, nz=64, n_detectors=8,
                                                 rays_per_detector=8192)
    phys = dp.create_physics()
    paths = dp.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    T = lambda a: torch.tensor(np.ascontiguousarray(a, np.float64).ravel(), device=paths.dev)
    f_true = paths.eval(T(truth), precision="fp64")[0].cpu().numpy()
    tau = 1e3 / np.median(f_true)
    counts = np.random.default_rng(5).poisson(tau * f_true)
    obs, W = counts / tau, tau * tau / np.maximum(counts, 1)
    rho0 = np.full(grid.ncell, 2650.0)
    prior = 1e-5
    rho1, hist = paths.solve(T(obs), T(rho0), method="gn", n_iter=1, weight=T(W), cg_iter=10,
                             precision="fp64", prior_weight=prior)
    L = _laplacian(grid.nx, grid.ny, grid.nz)
    J_of = lambda x: _device_jacobian(paths, T(x))[1]
    f_of = lambda x: paths.eval(T(x), precision="fp64")[0].cpu().numpy()
    ref, ref_hist = _gn_restated(J_of, f_of, obs, W, rho0, L, prior, n_iter=1)
    np.testing.assert_allclose(hist, ref_hist, rtol=1e-9)
    np.testing.assert_allclose(rho1.cpu().numpy(), ref, rtol=1e-8, atol=1e-6)
    assert hist[1] < hist[0]


def test_c5_gauss_newton_trajectory_against_oracle_loop(dp, oracle, orc_default):
    """Five Gauss-Newton iterations on a 32 x 32 x 16 grid (the C5 generator,
    2 detectors x 256 rays, Poisson counts ~10^3 per ray, prior 1e-5): the
    device loop (FP64) and the same loop driven by the oracle's forward model
    and per-ray Jacobian give the same misfit trajectory and the same density
    RMSE against the truth at every iteration."""
    import scipy.sparse as sp
    import torch
    from dpgpu.workloads import tomography_config
    grid, truth, rays, nodes = tomography_config(nx=32, ny=32, nz=16, n_detectors=2,
                                                 rays_per_detector=256, seed=77)
    tabs = [orc_default.table(i) for i in range(2)]
    phys = dp.upload_physics(tabs, ["StandardRock", "Air"])
    paths = dp.TomoPaths(phys, grid, rays, nodes, side_density=2500.0)
    T = lambda a: torch.tensor(np.ascontiguousarray(a, np.float64).ravel(), device=paths.dev)
    dims = np.array([grid.nx, grid.ny, grid.nz], np.int32)
    geom = np.array([*grid.origin, *grid.pitch])
    f_of = lambda x: oracle.tomo_forward(orc_default, 0, 1, dims, geom, x, 2500.0, rays, nodes)

    def J_of(x):
        rows, cols, vals = [], [], []
        for i, ray in enumerate(rays):
            _, cells, grads, _ = oracle.tomo_ray_grad(orc_default, 0, 1, dims, geom, x, 2500.0,
                                                      ray, nodes)
            rows.append(np.full(len(cells), i))
            cols.append(cells)
            vals.append(grads)
        J = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(len(rays), grid.ncell))
        J.sum_duplicates()
        return J

    f_true = f_of(truth.ravel())
    tau = 1e3 / np.median(f_true)
    counts = np.random.default_rng(6).poisson(tau * f_true)
    obs, W = counts / tau, tau * tau / np.maximum(counts, 1)
    rho0 = np.full(grid.ncell, 2650.0)
    prior = 1e-5
    L = _laplacian(grid.nx, grid.ny, grid.nz)
    ref, ref_hist = _gn_restated(J_of, f_of, obs, W, rho0, L, prior, n_iter=5)
    dev_rho, dev_hist = paths.solve(T(obs), T(rho0), method="gn", n_iter=5, weight=T(W),
                                    cg_iter=10, precision="fp64", prior_weight=prior)
    assert np.isfinite(ref_hist).all() and len(ref_hist) == 6
    np.testing.assert_allclose(dev_hist, ref_hist, rtol=1e-6)
    rmse = lambda x: float(np.sqrt(np.mean((x - truth.ravel()) ** 2)))
    assert rmse(dev_rho.cpu().numpy()) == pytest.approx(rmse(ref), rel=1e-6)
    np.testing.assert_allclose(dev_rho.cpu().numpy(), ref, rtol=1e-6, atol=1e-3)

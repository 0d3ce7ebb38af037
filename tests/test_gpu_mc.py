"""Stochastic backward MC on the GPU (straggled / mixed dual-mode transport)
against the oracle, through the C ABI.

Both sides transport over identical tables (the oracle's, Coulomb columns
included, uploaded with the elemental recipes) and draw from the same
counter-based Philox streams, so histories can be compared one by one.  In
FP64 the kernel evaluates the reference's operations; transcendental
functions (CUDA vs the host libm) differ in the last bit, so a history
agrees to ~1e-12 unless that difference flips a sampling decision, which
the tests allow for a small fraction of histories.  The mixed-precision
kernel is compared statistically (paired differences) and per history
with a looser bar.
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
def orc_phys(oracle):
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), coulomb=True)


@pytest.fixture(scope="module")
def phys(dp, orc_phys):
    tabs = [orc_phys.table(i) for i in range(3)]
    return dp.upload_physics(tabs, ["StandardRock", "Air", "Water"],
                             materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))


@pytest.fixture(scope="module")
def media(dp, phys):
    rock = dp.MaterialMixture(phys, 1)
    air = dp.MaterialMixture(phys, 2)
    mix = dp.MaterialMixture(phys, [1, 3, 2], [0.70, 0.25, 0.05])
    return rock, air, mix


def _agree(a, b, rtol):
    return np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)) + 1e-300


# ------------------------------------------------------------------ tables
def test_product_coulomb_tables_match_oracle(dp, orc_phys):
    """dp_physics_create builds the Coulomb scattering columns as
    create_physics(MUON) does (src/Physics.jl:386-397, src/Coulomb.jl:688-826)."""
    p = dp.create_physics(materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))
    for m in range(3):
        for c in ("lb1", "lbe", "mu0", "ecut", "fspin", "csda_R", "mixed_S", "xs"):
            a = p.column(m, c)
            b = orc_phys.column(m, "elastic_cutoff" if c == "ecut" else c)
            # mu0 is the root of a bracketing search with tolerances 1e-6
            # (src/Coulomb.jl:428-471): last-bit differences of its inputs
            # move it, and the paths derived from it, by up to ~1e-5
            rtol = 2e-5 if c in ("lb1", "lbe", "mu0", "ecut") else 1e-11
            np.testing.assert_allclose(a, b, rtol=rtol, atol=0, err_msg=f"{m} {c}")


# ------------------------------------------------------------------ kernel prep
@pytest.mark.parametrize("which", ["rock", "mixture"])
def test_mixed_kernel_matches_oracle(dp, media, oracle, orc_phys, which):
    """prepare_mixed_kernel (src/MixedTransport.jl:51-97) in the library
    against the oracle, single material and the rock/water/air mixture."""
    m = media[0] if which == "rock" else media[2]
    k = m.kernel()
    ref = oracle.mixed_kernel(orc_phys, [0]) if which == "rock" else \
        oracle.mixed_kernel(orc_phys, [0, 2, 1], [0.70, 0.25, 0.05])
    assert k["onset"] == ref["onset"]
    for a, b in (("energies", "E"), ("stopping", "stop"), ("sigma", "sigma"), ("range", "range"),
                 ("hazard", "hazard"), ("proper", "proper")):
        np.testing.assert_allclose(k[a], ref[b], rtol=1e-13, atol=0, err_msg=a)


# ------------------------------------------------------------------ histories
def _histories(n, seed, per_history_geometry=True):
    rng = np.random.default_rng(seed)
    E = np.exp(rng.uniform(np.log(1.0), np.log(1e4), n))
    q = np.where(rng.random(n) > 0.5, 1.0, -1.0)
    w = 2 * E * np.log(1e4)
    if per_history_geometry:
        t = rng.uniform(20.0, 500.0, n)
        geo = dict(thickness=t, density=rng.uniform(2000.0, 2800.0, n),
                   elevation=rng.uniform(30.0, 90.0, n), primary_altitude=t + 1000.0)
    else:
        geo = dict(thickness=120.0, density=2650.0, elevation=60.0, primary_altitude=1120.0)
    return E, q, w, geo


def _oracle_histories(oracle, orc_phys, E, q, w, geo, seed, rock=(0,), fracs=None, **kw):
    return oracle.mc_histories(orc_phys, list(rock), 1, geo["thickness"], geo["density"],
                               geo["elevation"], geo["primary_altitude"], E, q, w, seed=seed,
                               rock_fracs=fracs, **kw)


@pytest.mark.parametrize("case", ["straggled_scattering", "mixed_only", "mixture"])
def test_fp64_histories_match_oracle(dp, phys, media, oracle, orc_phys, case):
    """One history at a time: contribution, status, step count, final energy."""
    n, seed = 3000, 11
    E, q, w, geo = _histories(n, seed)
    rock, air, mix = media
    kw = dict(straggling=True, scattering=case != "mixed_only",
              threshold_low=100.0 if case != "mixed_only" else 1.0)
    if case == "mixture":
        oc, ost, osteps, oE = _oracle_histories(oracle, orc_phys, E, q, w, geo, seed, rock=(0, 2, 1),
                                                fracs=[0.70, 0.25, 0.05], **kw)
        med = mix
    else:
        oc, ost, osteps, oE = _oracle_histories(oracle, orc_phys, E, q, w, geo, seed, **kw)
        med = rock
    c, st, steps, Ef = dp.mc_histories(phys, med, air, E, q, w, seed=seed,
                                       straggling=kw["straggling"], scattering=kw["scattering"],
                                       energy_threshold_low=kw["threshold_low"], precision="fp64",
                                       **geo)
    assert np.all(st == 0) and np.all(ost == 0)
    same = _agree(c, oc, 1e-9) & (steps == osteps) & _agree(Ef[:, 0], oE, 1e-9)
    assert same.mean() >= 0.99, same.mean()
    assert (c > 0).sum() > n // 10  # a good share of histories reach the sky
    # estimator over all histories: paired difference within 3 sigma
    d = c - oc
    assert abs(d.mean()) <= 3 * d.std() / math.sqrt(n) + 1e-14 * abs(oc.mean())


def test_mixed_precision_histories_track_fp64(dp, phys, media, oracle, orc_phys):
    """FP32 transport (FP32 DCS sums and EHS angles, FP64 positions, DEL
    kinematics and tally) on the same random streams as the FP64 oracle: the
    paired flux difference is within 3 sigma of its own spread and below 1e-3
    of the flux.  Histories drift apart under the ~20 elastic deflections each
    samples from 24-bit uniforms, yet a large share still agrees to 1e-3."""
    n, seed = 20000, 5
    E, q, w, geo = _histories(n, seed)
    rock, air, mix = media
    oc, ost, _, _ = _oracle_histories(oracle, orc_phys, E, q, w, geo, seed, rock=(0, 2, 1),
                                      fracs=[0.70, 0.25, 0.05], straggling=True, scattering=True)
    c, st, _, _ = dp.mc_histories(phys, mix, air, E, q, w, seed=seed, precision="mixed", **geo)
    assert np.all(st == 0)
    d = c - oc
    f = oc.mean()
    assert abs(d.mean()) <= 3 * d.std() / math.sqrt(n) + 1e-12 * abs(f)
    assert abs(c.mean() - f) <= 1e-3 * abs(f) + 3 * d.std() / math.sqrt(n)
    assert _agree(c, oc, 1e-3).mean() >= 0.3
    assert abs((c > 0).mean() - (oc > 0).mean()) <= 0.01


# ------------------------------------------------------------------ batched LOS
def test_line_of_sight_batch_matches_oracle(dp, phys, media, oracle, orc_phys):
    """dp_mc_los: histories of all lines of sight in one launch; history id
    = running sample index; per-LOS flux and sigma from the compensated
    tally equal the oracle's over the same samples."""
    rock, air, _ = media
    depth = np.array([60.0, 150.0, 400.0])
    rho = np.array([2450.0, 2650.0, 2750.0])
    ns = np.array([300, 1000, 700])
    los = dp.make_los(ns, thickness=depth, density=rho, elevation=90.0, energy_min=1.0,
                      energy_max=1e4, primary_altitude=depth + 1000.0)
    out = dp.backward_mc_batch(phys, los, rock=rock, air=air, seed=3, precision="fp64",
                               scattering=False)
    E, q, w = dp.mc_samples(phys, energy_min=1.0, energy_max=1e4, n_samples=int(ns.sum()), seed=3)
    off = np.concatenate([[0], np.cumsum(ns)])
    for l in range(3):
        sl = slice(off[l], off[l + 1])
        oc, ost, _, _ = oracle.mc_histories(orc_phys, [0], 1, depth[l], rho[l], 90.0,
                                            depth[l] + 1000.0, E[sl], q[sl], w[sl], seed=3,
                                            id0=int(off[l]), straggling=True, scattering=False)
        f = oc.mean()
        s = math.sqrt(max((oc ** 2).mean() - f * f, 0.0) / ns[l])
        assert out["n_samples"][l] == ns[l] and out["n_status_nonzero"][l] == 0
        assert abs(out["flux"][l] - f) <= max(0.5 * s, 1e-9 * abs(f))
        assert out["sigma"][l] == pytest.approx(s, rel=0.05)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_line_of_sight_gradient_matches_oracle(dp, phys, media, oracle, orc_phys, precision):
    """compute_gradient over lines of sight: the CSDA sample-average flux and
    its derivative with respect to each line's density (src/Geometry.jl:933-945)
    over the stochastic run's own samples; mixed transport everywhere
    (threshold at the lowest final energy, no scattering).  FP64: the
    reference's operations; mixed: FP32 transport and tangent, FP64
    positions, within the 1e-4 mixed-mode bar."""
    rock, air, _ = media
    tol_f, tol_g = (1e-9, 1e-7) if precision == "fp64" else (1e-4, 1e-4)
    depth = np.array([50.0, 320.0, 1500.0])
    rho = np.array([2400.0, 2600.0, 2800.0])
    ns = np.array([64, 500, 256])
    los = dp.make_los(ns, thickness=depth, density=rho, elevation=90.0, energy_min=1.0,
                      energy_max=1e4)
    out = dp.backward_mc_batch(phys, los, rock=rock, air=air, seed=5, precision=precision,
                               scattering=False, energy_threshold_low=1.0, compute_gradient=True)
    E, q, w = dp.mc_samples(phys, energy_min=1.0, energy_max=1e4, n_samples=int(ns.sum()), seed=5)
    off = np.concatenate([[0], np.cumsum(ns)])
    for l in range(3):
        sl = slice(off[l], off[l + 1])
        cc, cd = oracle.backward_mc_csda(orc_phys, 0, 1, depth[l], rho[l], 90.0, E[sl], q[sl], w[sl])
        assert out["gradient_flux"][l] == pytest.approx(cc.mean(), rel=tol_f)
        assert out["gradient"][l] == pytest.approx(cd.mean(), rel=tol_g, abs=1e-12 * abs(cc.mean()))
        assert out["n_status_nonzero"][l] == 0 and out["flux"][l] > 0


def _philox_u01(ids, block, seed):
    """Philox4x32-10 (seed, (id, block)) -> two 53-bit uniforms per id."""
    M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
    c0 = ids.astype(np.uint64) & 0xFFFFFFFF
    c1 = ids.astype(np.uint64) >> 32
    c2 = np.full_like(c0, block)
    c3 = np.zeros_like(c0)
    k0, k1 = seed & 0xFFFFFFFF, seed >> 32
    for _ in range(10):
        p0, p1 = np.uint64(M0) * c0, np.uint64(M1) * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ np.uint64(k0)) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, \
            ((p0 >> 32) ^ c3 ^ np.uint64(k1)) & 0xFFFFFFFF, p0 & 0xFFFFFFFF
        k0, k1 = (k0 + W0) & 0xFFFFFFFF, (k1 + W1) & 0xFFFFFFFF
    f = lambda a, b: ((a >> 5).astype(np.float64) * 67108864.0 + (b >> 6).astype(np.float64)) \
        / 9007199254740992.0
    return f(c0, c1), f(c2, c3)


def test_drawn_geometry_batch_matches_oracle(dp, phys, media, oracle, orc_phys):
    """Per-history geometry drawn on the device (thickness U[20,500],
    density U[2000,2800] from Philox block 1, elevation U[30,90] from block 2,
    primary altitude thickness + 1000 m), the rock/water/air mixture."""
    rock, air, mix = media
    n, seed = 2000, 21
    los = dp.make_los(n, thickness=20.0, thickness_max=500.0, density=2000.0, density_max=2800.0,
                      elevation=30.0, elevation_max=90.0, air_height=1000.0, energy_min=1.0,
                      energy_max=1e4)
    out = dp.backward_mc_batch(phys, los, rock=mix, air=air, seed=seed, precision="fp64")
    ids = np.arange(n, dtype=np.uint64)
    u1, u2 = _philox_u01(ids, 1, seed)
    u3, _ = _philox_u01(ids, 2, seed)
    t = 20.0 + 480.0 * u1
    geo = dict(thickness=t, density=2000.0 + 800.0 * u2, elevation=30.0 + 60.0 * u3,
               primary_altitude=t + 1000.0)
    E, q, w = dp.mc_samples(phys, energy_min=1.0, energy_max=1e4, n_samples=n, seed=seed)
    oc, ost, _, _ = _oracle_histories(oracle, orc_phys, E, q, w, geo, seed, rock=(0, 2, 1),
                                      fracs=[0.70, 0.25, 0.05], straggling=True, scattering=True)
    f = oc.mean()
    s = math.sqrt(max((oc ** 2).mean() - f * f, 0.0) / n)
    assert out["n_status_nonzero"][0] == 0
    assert abs(out["flux"][0] - f) <= max(0.5 * s, 1e-9 * abs(f))


def test_run_backward_mc_stochastic(dp, phys, oracle, orc_phys):
    """run_backward_mc with straggling and scattering (the reference's
    defaults): flux and sigma of the stochastic transport, gradient of the
    CSDA surrogate over the same samples."""
    n = 3000
    kw = dict(rock_thickness=100.0, rock_density=2650.0, elevation=45.0, energy_min=1.0,
              energy_max=1e3, n_samples=n, seed=8)
    r = dp.run_backward_mc(phys, compute_gradient=True, **kw)
    E, q, w = dp.mc_samples(phys, energy_min=1.0, energy_max=1e3, n_samples=n, seed=8)
    oc, ost, _, _ = oracle.mc_histories(orc_phys, [0], 1, 100.0, 2650.0, 45.0, 3e4, E, q, w,
                                        seed=8, straggling=True, scattering=True)
    f = oc.mean()
    s = math.sqrt(max((oc ** 2).mean() - f * f, 0.0) / n)
    assert abs(r.flux - f) <= max(0.5 * s, 1e-9 * f)
    assert r.sigma == pytest.approx(s, rel=0.05)
    cc, cd = oracle.backward_mc_csda(orc_phys, 0, 1, 100.0, 2650.0, 45.0, E, q, w)
    assert r.gradient_flux == pytest.approx(cc.mean(), rel=1e-10)
    assert r.gradient == pytest.approx(cd.mean(), rel=1e-8)
    m = dp.run_backward_mc(phys, precision="mixed", **kw)
    assert abs(m.flux - r.flux) <= 3 * r.sigma


# ------------------------------------------------------------------ launch shapes
def test_cta_sizes_give_equivalent_histories(dp, phys, media):
    """A history's random stream is (seed, history id) whichever thread runs
    it.  Each compiled CTA size is its own instantiation, and the code
    generator fuses FP32 multiply-adds differently under different register
    budgets, so a history at 768 or 512 threads may take a rounding-flipped
    decision that it does not take at 1024: the sizes agree statistically
    (paired differences average to zero within 3 standard errors), not bit
    for bit.  At one size, every other launch choice gives identical bits
    (test_launch_shapes_give_identical_histories)."""
    n, seed = 20000, 5
    E, q, w, geo = _histories(n, seed)
    _, air, mix = media
    runs = {}
    try:
        for t in dp.mc_thread_choices("mixed"):
            dp.set_mc_threads(phys, "mc", "mixed", t)
            assert dp.get_mc_threads(phys, "mc", "mixed") == t
            c, st, _, _ = dp.mc_histories(phys, mix, air, E, q, w, seed=seed, precision="mixed",
                                          **geo)
            assert np.all(st == 0)
            runs[t] = c
    finally:
        dp.set_mc_threads(phys, "mc", "mixed", 0)
    assert dp.get_mc_threads(phys, "mc", "mixed") == 1024
    for t, c in runs.items():
        d = c - runs[1024]
        se = d.std() / math.sqrt(n)
        assert abs(d.mean()) <= 3 * se + 1e-15 * abs(runs[1024].mean()), (t, d.mean(), se)


def test_launch_shapes_give_identical_histories(dp, phys, media):
    """Table staging (shared memory or L1/L2) and the hand-out order (longest
    first or by index) do not change a result at one CTA size and lockstep
    mask: every shape gives the same contributions bit for bit, and histories
    taken out of order all end (none skipped or run twice).  The other
    lockstep masks (free-running phases, whose DCS sums are compiled
    separately and round differently in the last bits) agree statistically,
    and almost every history to 1e-4."""
    n, seed = 20000, 6
    E, q, w, geo = _histories(n, seed)
    _, air, mix = media
    assert dp.get_mc_shape(phys, "mc", "mixed") == {"threads": 1024, "staging": 1, "order": 0,
                                                     "sync": 3}  # the defaults
    runs = {}
    shapes = [(1024, 0, 0, 3), (1024, 0, 1, 3), (1024, 1, 0, 3), (1024, 1, 1, 3),
              (1024, 0, 0, 0), (1024, 0, 0, 1), (1024, 1, 1, 2)]
    try:
        for shape in shapes:
            dp.set_mc_shape(phys, "mc", "mixed", *shape)
            assert dp.get_mc_shape(phys, "mc", "mixed") == dict(zip(("threads", "staging",
                                                                     "order", "sync"), shape))
            c, st, ns, _ = dp.mc_histories(phys, mix, air, E, q, w, seed=seed,
                                           precision="mixed", **geo)
            assert np.all(st == 0) and np.all(ns > 0)
            runs[shape] = c
        with pytest.raises(ValueError):
            dp.set_mc_shape(phys, "mc", "mixed", 1024, 2, 0)
        with pytest.raises(ValueError):
            dp.set_mc_shape(phys, "mc", "mixed", 1024, 0, 2)
        with pytest.raises(ValueError):
            dp.set_mc_shape(phys, "mc", "mixed", 1024, 0, 0, 4)
    finally:
        dp.set_mc_shape(phys, "mc", "mixed", 0, 1, 0, 3)
    base = runs[shapes[0]]
    for shape, c in runs.items():
        if shape[3] == 3:
            np.testing.assert_array_equal(c, base, err_msg=str(shape))
        else:
            d = c - base
            assert abs(d.mean()) <= 3 * d.std() / math.sqrt(n) + 1e-15 * abs(base.mean()), shape
            assert np.mean(np.isclose(c, base, rtol=1e-4, atol=0.0)) > 0.98, shape


def test_autotune_shape_searches_every_dimension(dp, phys, media):
    """dp_autotune_shape: the CTA sizes, then the other staging, then the
    other order, then the other lockstep masks, each timed after an untimed
    run; the fastest shape stays on the context."""
    _, air, mix = media
    los = dp.make_los([4000], thickness=100.0, density=2650.0, elevation=60.0, energy_min=1.0,
                      energy_max=1e4, air_height=1000.0)
    calls = []

    def run():
        calls.append(1)
        dp.backward_mc_batch(phys, los, rock=mix, air=air, seed=1, precision="mixed")

    try:
        best, tried = dp.autotune_shape(phys, "mc", "mixed", run)
        n_sizes = len(dp.mc_thread_choices("mixed"))
        assert len(tried) == n_sizes + 1 + 1 + 3 and len(calls) == 2 * len(tried)
        assert {s["threads"] for s, _ in tried} == set(dp.mc_thread_choices("mixed"))
        assert {s["staging"] for s, _ in tried} == {0, 1}
        assert {s["order"] for s, _ in tried} == {0, 1}
        assert {s["sync"] for s, _ in tried} == {0, 1, 2, 3}
        assert all(v > 0 for _, v in tried)
        assert dp.get_mc_shape(phys, "mc", "mixed") == best
        assert best in [s for s, _ in tried]
    finally:
        dp.set_mc_shape(phys, "mc", "mixed", 0, 1, 0, 3)


def test_autotune_keeps_the_fastest_size(dp, phys, media):
    """dp_autotune runs the workload twice per compiled size (untimed, then
    timed), keeps the fastest on the context; a failing workload restores the
    previous size and raises."""
    _, air, mix = media
    los = dp.make_los([4000], thickness=100.0, density=2650.0, elevation=60.0, energy_min=1.0,
                      energy_max=1e4, air_height=1000.0)
    calls = []

    def run():
        calls.append(1)
        dp.backward_mc_batch(phys, los, rock=mix, air=air, seed=1, precision="mixed")

    choices = dp.mc_thread_choices("mixed")
    try:
        best, ms = dp.autotune(phys, "mc", "mixed", run)
        assert best in choices and sorted(ms) == sorted(choices)
        assert all(v > 0 for v in ms.values()) and ms[best] == min(ms.values())
        assert dp.get_mc_threads(phys, "mc", "mixed") == best
        assert len(calls) == 2 * len(choices)
        dp.set_mc_threads(phys, "mc", "mixed", 768)

        def broken():
            raise RuntimeError("workload failed")

        with pytest.raises(RuntimeError, match="workload failed"):
            dp.autotune(phys, "mc", "mixed", broken)
        assert dp.get_mc_threads(phys, "mc", "mixed") == 768
        with pytest.raises(ValueError):
            dp.set_mc_threads(phys, "mc", "mixed", 640)
        with pytest.raises(ValueError):
            dp.set_mc_threads(phys, "mc", "fp64", 512)
    finally:
        dp.set_mc_threads(phys, "mc", "mixed", 0)


# ------------------------------------------------------------------ porous layer
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_porous_layer_batch_matches_oracle(dp, phys, media, oracle, orc_phys, precision):
    """dp_mc_los_layers: the shallow porous top layer of TwoLayerGeometry
    (src/Geometry.jl:617-635; here water at 1000 kg/m^3 over the top 25-60 m
    of rock) against the oracle's histories on the same streams: FP64 per line
    of sight within 0.5 sigma (to 1e-9 when no history flips), mixed
    precision within 3 sigma.  A zero-thickness layer is no layer (the
    porous kernel is compiled apart, so to within its sigma, not bitwise)."""
    rock, air, _ = media
    water = dp.MaterialMixture(phys, 3)
    depth = np.array([60.0, 150.0, 400.0])
    pt = np.array([25.0, 60.0, 40.0])
    ns = np.array([400, 800, 600])
    kw = dict(thickness=depth, density=2650.0, elevation=70.0, energy_min=1.0, energy_max=1e4,
              air_height=1000.0)
    los = dp.make_los(ns, porous_thickness=pt, porous_density=1000.0, **kw)
    out = dp.backward_mc_batch(phys, los, rock=rock, air=air, porous=water, seed=3,
                               precision=precision, scattering=True)
    E, q, w = dp.mc_samples(phys, energy_min=1.0, energy_max=1e4, n_samples=int(ns.sum()), seed=3)
    off = np.concatenate([[0], np.cumsum(ns)])
    for l in range(3):
        sl = slice(off[l], off[l + 1])
        oc, ost, _, _ = oracle.mc_histories(orc_phys, [0], 1, depth[l], 2650.0, 70.0,
                                            depth[l] + 1000.0, E[sl], q[sl], w[sl], seed=3,
                                            id0=int(off[l]), porous=2, porous_thickness=pt[l],
                                            porous_density=1000.0)
        assert np.all(ost == 0)
        f = oc.mean()
        s = math.sqrt(max((oc ** 2).mean() - f * f, 0.0) / ns[l])
        assert out["n_status_nonzero"][l] == 0
        bar = max(0.5 * s, 1e-9 * abs(f)) if precision == "fp64" else 3 * s + 1e-3 * abs(f)
        assert abs(out["flux"][l] - f) <= bar, (l, out["flux"][l], f, s)
    plain = dp.backward_mc_batch(phys, dp.make_los(ns, **kw), rock=rock, air=air, seed=3,
                                 precision=precision, scattering=True)
    zero = dp.backward_mc_batch(phys, dp.make_los(ns, porous_thickness=0.0, porous_density=1000.0,
                                                  **kw),
                                rock=rock, air=air, porous=water, seed=3, precision=precision,
                                scattering=True)
    # a layer of zero thickness runs the porous kernel, a separate instantiation
    # of the transport: in FP64 it follows the plain kernel's histories; in
    # mixed precision its FP32 roundings (fused multiply-adds) can differ, so
    # the two estimates agree statistically
    tol = 0.5 if precision == "fp64" else 3.0
    assert np.all(np.abs(zero["flux"] - plain["flux"]) <= tol * plain["sigma"] + 1e-12)
    assert np.all(out["flux"] > plain["flux"])
    with pytest.raises(ValueError):
        dp.backward_mc_batch(phys, los, rock=rock, air=air, porous=water, compute_gradient=True)


def test_compute_flux_with_porous_layer(dp, phys, oracle, orc_phys):
    """compute_flux (src/Geometry.jl:899-929) with porous_* keywords: in CSDA
    mode (straggling = scattering = false) the estimate is deterministic
    given the samples and equals the oracle's to 1e-10; with straggling and
    scattering it agrees within 3 sigma."""
    n = 2000
    kw = dict(n_samples=n, seed=11, porous_material=3, porous_density=1000.0,
              porous_thickness=20.0)
    f, s = dp.compute_flux(phys, 2650.0, 80.0, 55.0, 1.0, 50.0, straggling=False,
                           scattering=False, **kw)
    E, q, w = dp.mc_samples(phys, energy_min=1.0, energy_max=50.0, n_samples=n, seed=11)
    oc, ost, _, _ = oracle.mc_histories(orc_phys, [0], 1, 80.0, 2650.0, 55.0, 3e4, E, q, w,
                                        seed=11, straggling=False, scattering=False, porous=2,
                                        porous_thickness=20.0, porous_density=1000.0)
    assert np.all(ost == 0)
    assert f == pytest.approx(oc.mean(), rel=1e-10)
    assert s == pytest.approx(math.sqrt(max((oc ** 2).mean() - oc.mean() ** 2, 0.0) / n),
                              rel=1e-8)
    f2, s2 = dp.compute_flux(phys, 2650.0, 80.0, 55.0, 1.0, 50.0, **kw)
    oc2, _, _, _ = oracle.mc_histories(orc_phys, [0], 1, 80.0, 2650.0, 55.0, 3e4, E, q, w,
                                       seed=11, porous=2, porous_thickness=20.0,
                                       porous_density=1000.0)
    assert abs(f2 - oc2.mean()) <= 3 * s2
    with pytest.raises(ValueError):
        dp.compute_flux(phys, 2650.0, 80.0, 55.0, 1.0, 50.0, porous_material=3,
                        porous_thickness=20.0, porous_density=0.0)


def test_flux_uncertainty_budget(dp):
    """test/runtests.jl:222-245 on the device: compute_flux_uncertainty with
    create_physics(n_energies=30, K_min=0.05, K_max=1e4); every variation
    reuses the nominal seed (common random numbers)."""
    physics = dp.create_physics(n_energies=30, K_min=0.05, K_max=1e4)
    b = dp.compute_flux_uncertainty(physics, 2650.0, 25.0, 55.0, 1.0, 50.0, n_samples=8,
                                    seed=11, straggling=True, scattering=True,
                                    energy_threshold_low=50.0, threshold_factors=(0.5, 2.0))
    for v in (b.value, b.sigma_mc, b.sigma_syst, b.sigma_total):
        assert math.isfinite(v)
    assert b.sigma_mc >= 0.0 and b.sigma_syst >= 0.0
    assert b.sigma_total >= b.sigma_mc and b.sigma_total >= b.sigma_syst
    assert len(b.sources["energy_threshold_low"].variant_values) == 2
    f, s = dp.compute_flux(physics, 2650.0, 25.0, 55.0, 1.0, 50.0, n_samples=8, seed=11,
                           energy_threshold_low=50.0)
    assert (b.value, b.sigma_mc) == (f, s)

"""Fixed-path stochastic MC on the GPU (compute_directional_flux_mc,
src/Tomography.jl:826-1041) against the oracle, through the C ABI.

Both sides use identical tables and the same Philox streams (history i of a
batch: stream (seed, i)), so histories compare one by one in FP64; the
mixed-precision kernel is compared statistically."""
import math

import numpy as np
import pytest

from test_gpu_mc import _agree, _philox_u01

pytestmark = pytest.mark.gpu

DET_ELEV = 963.0
PRIMARY = 3e4


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
def scene(dp, phys):
    """A voxel column of 24 cells with water fractions 0 and 0.3 (two
    mixtures), six directions crossing 3-12 cells each, rock beyond the
    cells and air to 30 km above a detector at 963 m."""
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2710.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(DET_ELEV, PRIMARY)
    wf = np.where(np.arange(24) % 3 == 1, 0.3, 0.0)
    mats, dens = dp.build_cell_properties_for_mc(phys, np.zeros(24, bool), wf, cfg)
    rng = np.random.default_rng(7)
    paths = []
    for d, zen in enumerate((0.0, 25.0, 40.0, 55.0, 65.0, 75.0)):
        k = 3 + (d * 7) % 10
        cells = rng.choice(24, size=k, replace=False) + 1
        segs = [dp.CellSegment(int(c), float(rng.uniform(4.0, 30.0))) for c in cells]
        paths.append(dp.DirectionalPath(zen, 0.0, segs, 0.0, 0.0, float(rng.uniform(0.0, 400.0)),
                                        float(rng.uniform(80.0, 300.0)), True))
    return cfg, site, mats, dens, paths


def _samples(n_per, seed, emin=0.5, emax=1e5):
    rng = np.random.default_rng(seed)
    out = []
    for n in n_per:
        E = np.exp(rng.uniform(math.log(emin), math.log(emax), n))
        q = np.where(rng.random(n) > 0.5, 1.0, -1.0)
        out.append([(e, c, e * math.log(emax / emin)) for e, c in zip(E, q)])
    return out


def _oracle_batch(dp, oracle, orc_phys, scene, samples, seed, straggling=True, low=100.0):
    """The same batch on the oracle: media in the product's order (cell
    mixtures by use, rock, air)."""
    cfg, site, mats, dens, paths = scene
    use = {}
    for p, ss in zip(paths, samples):
        for s in p.segments:
            m = mats[s.cell_idx - 1]
            use[id(m)] = (m, use.get(id(m), (m, 0))[1] + len(ss))
    uniq = [m for m, _ in sorted(use.values(), key=lambda t: -t[1])]
    media = [([a - 1 for a in u.materials], u.fractions) for u in uniq]
    media += [([cfg.rock_material - 1], [1.0]), ([cfg.air_material - 1], [1.0])]
    index = {id(u): k for k, u in enumerate(uniq)}
    seg_ptr = np.zeros(len(paths) + 1, np.int64)
    sm, sd, sl = [], [], []
    for d, p in enumerate(paths):
        seg_ptr[d + 1] = seg_ptr[d] + len(p.segments)
        for s in p.segments:
            sm.append(index[id(mats[s.cell_idx - 1])])
            sd.append(dens[s.cell_idx - 1])
            sl.append(s.distance)
    cos_t = np.array([math.cos(math.radians(p.zenith)) for p in paths])
    air = np.array([max(0.0, PRIMARY - p.surface_exit_z) / max(c, 1e-3)
                    for p, c in zip(paths, cos_t)])
    smp_ptr = np.concatenate([[0], np.cumsum([len(s) for s in samples])])
    E = np.array([s[0] for ss in samples for s in ss])
    q = np.array([s[1] for ss in samples for s in ss])
    w = np.array([s[2] for ss in samples for s in ss])
    return oracle.dir_histories(orc_phys, media, len(media) - 2, cfg.rock_density,
                                len(media) - 1, DET_ELEV, cos_t,
                                [p.remaining_rock_distance for p in paths], air, seg_ptr,
                                np.array(sm, np.int32), sd, sl, smp_ptr, E, q, w, seed=seed,
                                straggling=straggling, threshold_low=low, energy_limit=1e9)


def _run(dp, phys, scene, samples, seed, **kw):
    cfg, site, mats, dens, paths = scene
    es = [[dp.EnergySample(*s) for s in ss] for ss in samples]
    return dp.directional_flux_mc_batch(phys, cfg, site, paths, mats, dens, es, seed,
                                        return_histories=True, **kw)


def _tally(c, n_per):
    off = np.concatenate([[0], np.cumsum(n_per)])
    f, s = [], []
    for a, b in zip(off[:-1], off[1:]):
        n = b - a
        x = c[a:b]
        m = x.sum() / max(n, 1)
        f.append(m)
        s.append(math.sqrt(max(0.0, ((x ** 2).sum() / max(n, 1) - m * m) / max(1, n - 1))))
    return np.array(f), np.array(s)


@pytest.mark.parametrize("straggling", [True, False])
def test_fp64_histories_match_oracle(dp, phys, oracle, orc_phys, scene, straggling):
    """One history at a time: 2 w_i w flux_i and status; per direction the
    tally's flux and sigma (n - 1 form)."""
    n_per = [400, 300, 500, 350, 450, 300]
    samples = _samples(n_per, 3)
    seed = 31
    oc, ost, _, _ = _oracle_batch(dp, oracle, orc_phys, scene, samples, seed, straggling)
    r = _run(dp, phys, scene, samples, seed, straggling=straggling, precision="fp64")
    assert np.all(ost == 0) and np.all(r["status"] == 0)
    assert np.all(r["n_status_nonzero"] == 0)
    same = _agree(r["contrib"], oc, 1e-9)
    assert same.mean() >= (0.99 if straggling else 1.0), same.mean()
    assert (oc > 0).sum() > len(oc) // 10
    f, s = _tally(oc, n_per)
    if straggling:
        d = r["contrib"] - oc
        assert abs(d.mean()) <= 3 * d.std() / math.sqrt(len(d)) + 1e-14 * abs(oc.mean())
    else:
        np.testing.assert_allclose(r["flux"], f, rtol=1e-10)
        np.testing.assert_allclose(r["sigma"], s, rtol=1e-8)
    np.testing.assert_array_equal(r["n_samples"], n_per)


def test_mixed_precision_tracks_fp64(dp, phys, oracle, orc_phys, scene):
    """FP32 transport on the same streams: per direction the flux agrees with
    the FP64 oracle within 3 sigma of the paired differences."""
    n_per = [3000] * 6
    samples = _samples(n_per, 4)
    seed = 32
    oc, ost, _, _ = _oracle_batch(dp, oracle, orc_phys, scene, samples, seed)
    r = _run(dp, phys, scene, samples, seed, precision="mixed")
    assert np.all(r["status"] == 0)
    off = np.concatenate([[0], np.cumsum(n_per)])
    for d, (a, b) in enumerate(zip(off[:-1], off[1:])):
        x, y = r["contrib"][a:b], oc[a:b]
        diff = x - y
        n = b - a
        f = y.mean()
        assert abs(diff.mean()) <= 3 * diff.std() / math.sqrt(n) + 1e-3 * abs(f), d
        assert r["flux"][d] == pytest.approx(x.mean(), rel=1e-12)


def test_invalid_paths_and_empty_directions(dp, phys, scene):
    """An invalid path (or cos zenith <= 0) gives (NaN, NaN)
    (src/Tomography.jl:991-993); a direction with no samples gives (0, 0)."""
    cfg, site, mats, dens, paths = scene
    bad = paths[1]._replace(valid=False)
    down = paths[2]._replace(zenith=95.0)
    ps = [paths[0], bad, down, paths[3]]
    samples = _samples([50, 50, 50, 0], 5)
    es = [[dp.EnergySample(*s) for s in ss] for ss in samples]
    r = dp.directional_flux_mc_batch(phys, cfg, site, ps, mats, dens, es, 9, precision="mixed")
    assert np.isfinite(r["flux"][0]) and r["flux"][0] > 0
    assert np.isnan(r["flux"][1]) and np.isnan(r["sigma"][1])
    assert np.isnan(r["flux"][2]) and np.isnan(r["sigma"][2])
    assert r["flux"][3] == 0.0 and r["sigma"][3] == 0.0


def test_drawn_samples_match_oracle(dp, phys, oracle, orc_phys, scene):
    """Energies and charges drawn on the device (Philox block 0:
    sample_energy_set semantics) equal the explicit samples of the same
    draws."""
    n_per = [256] * 6
    seed = 33
    emin, emax = 1e-3, 1e9
    ids = np.arange(sum(n_per), dtype=np.uint64)
    u1, u2 = _philox_u01(ids, 0, seed)
    rk = math.log(emax / emin)
    E = emin * np.exp(rk * u1)
    q = np.where(u2 > 0.5, 1.0, -1.0)
    off = np.concatenate([[0], np.cumsum(n_per)])
    samples = [[(E[i], q[i], E[i] * rk) for i in range(a, b)] for a, b in zip(off[:-1], off[1:])]
    cfg, site, mats, dens, paths = scene
    drawn = dp.directional_flux_mc_batch(phys, cfg, site, paths, mats, dens, None, seed,
                                         n_samples=n_per, energy_min=emin, energy_max=emax,
                                         precision="fp64", return_histories=True)
    given = _run(dp, phys, scene, samples, seed, precision="fp64")
    np.testing.assert_allclose(drawn["contrib"], given["contrib"], rtol=1e-12, atol=0)
    oc, _, _, _ = _oracle_batch(dp, oracle, orc_phys, scene, samples, seed)
    assert _agree(drawn["contrib"], oc, 1e-9).mean() >= 0.99


def test_single_direction_api(dp, phys, oracle, orc_phys, scene):
    """compute_directional_flux_mc for one path: the batch form's result for
    that path, and the oracle's flux within its sigma."""
    cfg, site, mats, dens, paths = scene
    samples = _samples([500], 6)
    es = [dp.EnergySample(*s) for s in samples[0]]
    f, s = dp.compute_directional_flux_mc(phys, cfg, site, paths[4], mats, dens, es, 41,
                                          straggling=True, energy_threshold_low=100.0)
    r = dp.directional_flux_mc_batch(phys, cfg, site, [paths[4]], mats, dens, [es], 41,
                                     precision="fp64")
    assert f == r["flux"][0] and s == r["sigma"][0]
    sub = (cfg, site, mats, dens, [paths[4]])
    oc, _, _, _ = _oracle_batch(dp, oracle, orc_phys, sub, samples, 41)
    fo, so = _tally(oc, [500])
    assert f > 0 and abs(f - fo[0]) <= max(so[0], 1e-9 * fo[0])


def test_cta_sizes_give_equivalent_histories(dp, phys, scene):
    """Fixed-path transport at every compiled CTA size (fewer media fit in
    shared memory at larger sizes): a history's stream does not depend on
    the thread that runs it, but each size is its own instantiation whose
    FP32 multiply-adds the code generator may fuse differently, so the sizes
    agree statistically (paired differences within 3 standard errors) and
    mostly bit for bit."""
    n_per = [2000] * 6
    samples = _samples(n_per, 9)
    runs = {}
    try:
        for t in dp.mc_thread_choices("mixed"):
            dp.set_mc_threads(phys, "dir", "mixed", t)
            r = _run(dp, phys, scene, samples, 33, precision="mixed")
            assert np.all(r["status"] == 0)
            runs[t] = r
    finally:
        dp.set_mc_threads(phys, "dir", "mixed", 0)
    ref = runs[1024]["contrib"]
    for t, r in runs.items():
        d = r["contrib"] - ref
        se = d.std() / math.sqrt(len(d))
        assert abs(d.mean()) <= 3 * se + 1e-15 * abs(ref.mean()), (t, d.mean(), se)

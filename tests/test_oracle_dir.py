"""The oracle's fixed-path MC (compute_directional_flux_mc and its segment
propagation, src/Tomography.jl:826-1041) against the reference's own
known-answer tests (test/test_mixed_kernel.jl:85-185), and the host-side
checks of the product's fixed-path API (CPU only)."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def phys32(oracle):
    """create_physics(MUON; n_energies=32, K_min=1e-3, K_max=1e6, [rock, air, water])."""
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), n=32,
                                  Kmin=1e-3, Kmax=1e6, coulomb=True)


@pytest.mark.parametrize("remaining", [2e-8, 5e-7, 1e-6, 1e-4])
def test_segment_step_never_overshoots(oracle, remaining):
    """test/test_mixed_kernel.jl:179-184: 0 < step <= remaining."""
    for max_step in (1e-10, remaining / 2, 1.0):
        step = oracle.mc_segment_step(remaining, max_step)
        assert 0.0 < step <= remaining


def test_segment_conserves_distance_and_grammage(oracle, phys32):
    """test/test_mixed_kernel.jl:101-106: a 100 m rock segment at 2650 kg/m^3
    from 99 GeV (straggled steps, then mixed steps above 100 GeV) travels
    100 m and 265000 kg/m^2."""
    uz = -math.cos(math.radians(20.0))
    for seed in (17, 18, 19):
        s, st, _ = oracle.dir_segment(phys32, [0], dict(energy=99.0, uz=uz), 2650.0, 100.0,
                                      straggling=True, threshold_low=100.0, energy_limit=1e6,
                                      seed=seed)
        assert st == 0
        assert s["distance"] == pytest.approx(100.0, abs=1e-8)
        assert s["grammage"] == pytest.approx(265000.0, abs=1e-5)
        assert s["z"] == pytest.approx(100.0 * math.cos(math.radians(20.0)), rel=1e-12)


def test_zero_increment_at_mode_change(oracle):
    """test/test_mixed_kernel.jl:147-163: a straggled step from prevfloat(100)
    that reaches the mode switch after a sub-ulp displacement is progress; the
    rest of the 1 mm segment is then consumed by the mixed step."""
    p = oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR), n=12, Kmin=1.0, Kmax=1e6,
                               coulomb=True)
    E0 = float(np.nextafter(100.0, 0.0))
    s, st, used = oracle.dir_segment(p, [0], dict(energy=E0, distance=1000.0), 2650.0, 0.001,
                                     straggling=True, threshold_low=100.0, energy_limit=1e6,
                                     script=[1e-12, 0.5, 1e10, 1e10])
    assert st == 0
    assert s["energy"] >= 100.0
    assert s["distance"] - 1000.0 == pytest.approx(0.001, abs=4 * np.spacing(1000.0))
    assert s["grammage"] == pytest.approx(2.65, rel=1e-10)


def _one_path(cos_t, lengths, remaining=0.0, air=0.0):
    lengths = np.atleast_1d(lengths)
    return dict(cos_theta=[cos_t], remaining_rock=[remaining], air_distance=[air],
                seg_ptr=[0, len(lengths)], seg_medium=np.zeros(len(lengths), np.int32),
                seg_density=np.full(len(lengths), 2650.0), seg_length=lengths)


def test_csda_single_sample_flux(oracle, phys32):
    """test/test_mixed_kernel.jl:92-100: straggling off, one sample at 1 TeV
    through 100 m of rock at 20 deg and air to 12 km: flux > 0, sigma = 0."""
    ct = math.cos(math.radians(20.0))
    path = _one_path(ct, [100.0], air=max(0.0, 12000.0 - 60.0) / max(ct, 1e-3))
    c, st, _, _ = oracle.dir_histories(phys32, [([0], [1.0]), ([1], [1.0])], 0, 2650.0, 1, 1000.0,
                                       smp_ptr=[0, 1], E=[1000.0], q=[1.0], w=[1.0], seed=42,
                                       straggling=False, energy_limit=1e6, **path)
    n = 1
    flux = c.sum() / n
    var = ((c ** 2).sum() / n - flux ** 2) / max(1, n - 1)
    assert st[0] == 0 and flux > 0 and math.isfinite(flux)
    assert math.sqrt(max(0.0, var)) == 0.0


def test_segments_split_equals_one_segment_csda(oracle, phys32):
    """Deterministic transport: a column cut into cells of one medium gives the
    flux of the uncut column to rounding (the 1 %-range step rule restarts at
    each cell boundary, so only to 1e-4)."""
    ct = math.cos(math.radians(30.0))
    E = np.array([3.0, 30.0, 300.0, 3000.0])
    kw = dict(smp_ptr=[0, 4], E=E, q=np.ones(4), w=np.ones(4), seed=1, straggling=False,
              energy_limit=1e6)
    media = [([0], [1.0]), ([1], [1.0])]
    a, _, _, _ = oracle.dir_histories(phys32, media, 0, 2650.0, 1, 963.0,
                                      **_one_path(ct, [200.0], air=3e4 / ct), **kw)
    b, _, _, _ = oracle.dir_histories(phys32, media, 0, 2650.0, 1, 963.0,
                                      **_one_path(ct, [50.0] * 4, air=3e4 / ct), **kw)
    assert np.all(a > 0)
    np.testing.assert_allclose(b, a, rtol=1e-4)


def test_api_rejects_scattering_and_quadrature_nodes():
    """The reference's ArgumentErrors (src/Tomography.jl:987-990), raised on
    the host before any device work."""
    import dpgpu
    cfg = dpgpu.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dpgpu.SiteConfig(1000.0, 12000.0)
    path = dpgpu.DirectionalPath(20.0, 0.0, [dpgpu.CellSegment(1, 100.0)], 100.0, 100.0, 0.0,
                                 60.0, True)
    samples = [dpgpu.EnergySample(1000.0, 1.0, 1.0)]
    with pytest.raises(ValueError):
        dpgpu.compute_directional_flux_mc(None, cfg, site, path, [], [2650.0], samples, 42,
                                          straggling=True, energy_threshold_low=100.0,
                                          scattering=True)
    with pytest.raises(ValueError):
        dpgpu.compute_directional_flux_mc(None, cfg, site, path, [], [2650.0],
                                          [dpgpu.EnergySample(1000.0, 0.0, 1.0)], 42,
                                          straggling=True, energy_threshold_low=100.0)


def test_cell_mixture_and_density():
    """mc_cell_mixture_and_density (src/Tomography.jl:826-845): specific
    volumes add; w <= 1e-12 is pure rock; the porous top layer splits the
    non-water mass evenly."""
    import dpgpu
    cfg = dpgpu.MaterialConfig(1, 3, 2, 4, 2650.0, 1000.0, 1800.0, 20.0)
    (m, f), rho = dpgpu.mc_cell_mixture_and_density(0.0, False, cfg)
    assert m == (1,) and f == (1.0,) and rho == 2650.0
    (m, f), rho = dpgpu.mc_cell_mixture_and_density(0.3, False, cfg)
    assert m == (1, 3) and f == (0.7, 0.3)
    assert rho == pytest.approx(1.0 / (0.7 / 2650.0 + 0.3 / 1000.0), rel=1e-15)
    (m, f), rho = dpgpu.mc_cell_mixture_and_density(0.2, True, cfg)
    assert m == (4, 1, 3) and f == pytest.approx((0.4, 0.4, 0.2))
    assert rho == pytest.approx(1.0 / (0.4 / 1800.0 + 0.4 / 2650.0 + 0.2 / 1000.0), rel=1e-15)


def test_shallow_porous_recipe_and_guards():
    """test/test_shallow_mixture.jl: the shallow porous cell is 1/2 (1 - w)
    rock, w water, 1/2 (1 - w) porous with harmonic density, down to w = 0
    (the pure-rock shortcut belongs to the ordinary branch); either guard
    (no porous material, no porous top thickness) or a deep cell disables it."""
    import dpgpu
    cfg = dpgpu.MaterialConfig(1, 2, 3, 3, 2700.0, 1000.0, 1500.0, 50.0)
    for w in (0.0, 5e-13, 1e-12, 2e-12, 1e-8, 0.3, 1.0):
        (mats, fr), rho = dpgpu.mc_cell_mixture_and_density(w, True, cfg)
        share = dict(zip(mats, fr))
        expected = {1: 0.5 * (1 - w), 2: w, 3: 0.5 * (1 - w)}  # rock, water, porous
        assert share == pytest.approx(expected, rel=2e-15, abs=0)
        assert rho == pytest.approx(1 / (0.5 * (1 - w) / 2700 + w / 1000 + 0.5 * (1 - w) / 1500),
                                    rel=2e-15)
    for shallow, c in ((False, cfg), (True, cfg._replace(porous_material=0)),
                       (True, cfg._replace(porous_top_thickness=0.0))):
        for w in (0.0, 5e-13, 0.3):
            (mats, fr), rho = dpgpu.mc_cell_mixture_and_density(w, shallow, c)
            ew = 0.0 if w <= 1e-12 else w
            assert rho == pytest.approx(1 / ((1 - ew) / 2700 + ew / 1000), rel=2e-15)
            assert 3 not in mats

"""Transport-systematic uncertainty budgets (src/Uncertainty.jl) on the CPU:
the budget algebra pinned to the reference's known answers
(test/runtests.jl:156-220)."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


def test_budget_combination_math(dp):
    """test/runtests.jl:157-182: a vector observable whose variations shift
    it by known amounts."""
    def evaluator(v):
        base = (2.0 if v.straggling else 0.0) + (3.0 if v.scattering else 0.0) + \
            v.energy_threshold_low / 10.0
        return np.array([100.0 + base, 200.0 + 2.0 * base]), np.array([0.25, 0.50])

    b = dp.estimate_transport_uncertainty(evaluator, straggling=True, scattering=True,
                                          energy_threshold_low=10.0, seed=7,
                                          threshold_factors=(0.5, 2.0))
    np.testing.assert_allclose(b.value, [106.0, 212.0])
    np.testing.assert_allclose(b.sigma_mc, [0.25, 0.50])
    np.testing.assert_allclose(b.sources["straggling"].sigma, [2.0, 4.0])
    np.testing.assert_allclose(b.sources["scattering"].sigma, [3.0, 6.0])
    np.testing.assert_allclose(b.sources["energy_threshold_low"].sigma, [1.0, 2.0])
    np.testing.assert_allclose(b.sigma_syst, np.sqrt([14.0, 56.0]))
    np.testing.assert_allclose(b.sigma_total, np.sqrt([14.0 + 0.25 ** 2, 56.0 + 0.50 ** 2]))
    assert b.sources["energy_threshold_low"].variant_labels == ["threshold=5.0",
                                                               "threshold=20.0"]
    assert b.sources["straggling"].variant_labels == ["straggling=false"]
    assert b.nominal == dp.TransportVariation(True, True, 10.0, 7)


def test_same_seed_evaluation_is_deterministic(dp):
    """test/runtests.jl:184-220: a seeded evaluator gives identical budgets."""
    def evaluator(v):
        rng = np.random.default_rng(v.seed)
        value = 1.0 + (0.3 if v.straggling else -0.2) + (0.5 if v.scattering else -0.4) + \
            v.energy_threshold_low / 100.0 + rng.random()
        return value, rng.random() / 10.0

    kw = dict(straggling=True, scattering=True, energy_threshold_low=20.0, seed=17,
              threshold_factors=(0.5, 2.0))
    a = dp.estimate_transport_uncertainty(evaluator, **kw)
    b = dp.estimate_transport_uncertainty(evaluator, **kw)
    assert (a.value, a.sigma_mc, a.sigma_syst, a.sigma_total) == \
        (b.value, b.sigma_mc, b.sigma_syst, b.sigma_total)
    assert a.sources["straggling"].variant_values == b.sources["straggling"].variant_values
    assert a.sources["energy_threshold_low"].variant_values == \
        b.sources["energy_threshold_low"].variant_values
    assert isinstance(a.value, float) and isinstance(a.sigma_total, float)


def test_threshold_variants_and_relative_percent(dp):
    """Duplicate, non-positive and nominal-equal factors are dropped
    (src/Uncertainty.jl:79-103); relative_uncertainty_percent guards the
    denominator (:230-237)."""
    calls = []

    def evaluator(v):
        calls.append(v.energy_threshold_low)
        return 1.0, 0.0

    b = dp.estimate_transport_uncertainty(evaluator, energy_threshold_low=50.0,
                                          threshold_factors=(0.5, 1.0, 0.5, -1.0, 1 + 1e-12,
                                                             2.0))
    assert b.sources["energy_threshold_low"].variant_labels == ["threshold=25.0",
                                                               "threshold=100.0"]
    assert calls == [50.0, 50.0, 50.0, 25.0, 100.0]
    b0 = dp.estimate_transport_uncertainty(evaluator, energy_threshold_low=0.0)
    assert b0.sources["energy_threshold_low"].variant_values == []
    assert dp.relative_uncertainty_percent(2.0, 0.1) == pytest.approx(5.0)
    assert dp.relative_uncertainty_percent(0.0, 1e-31) == pytest.approx(10.0)
    np.testing.assert_allclose(dp.relative_uncertainty_percent([4.0, -2.0], [1.0, 1.0]),
                               [25.0, 50.0])

"""Transport-systematic uncertainty budgets (src/Uncertainty.jl).

estimate_transport_uncertainty evaluates an observable at the nominal
transport settings and at one-at-a-time variations (straggling toggled,
scattering toggled, the mode-switch threshold scaled), takes per source the
envelope of |variant - nominal| and combines the sources and the MC error in
quadrature.  compute_flux_uncertainty does this for compute_flux with common
random numbers: every variation reuses the nominal seed, so the device draws
the same final energies and charges for each (Philox streams keyed by the
seed and the sample index).
"""
import math
from collections import namedtuple

import numpy as np

PRIMARY_ALTITUDE = 3e4

# src/Uncertainty.jl:27-57
TransportVariation = namedtuple("TransportVariation",
                                "straggling scattering energy_threshold_low seed")
SystematicSourceResult = namedtuple("SystematicSourceResult",
                                    "sigma reference_value variant_values variant_sigmas "
                                    "variant_labels")
TransportUncertaintyResult = namedtuple("TransportUncertaintyResult",
                                        "value sigma_mc sigma_syst sigma_total sources nominal")


def _zero_like(x):
    return np.zeros_like(x, dtype=np.float64) if isinstance(x, np.ndarray) else 0.0


def _as_value(x):
    """Scalars stay floats, arrays become float64 arrays."""
    if np.ndim(x) == 0:
        return float(x)
    return np.asarray(x, np.float64)


def _evaluate_source(evaluate, nominal_value, variants, labels):
    """_evaluate_source (src/Uncertainty.jl:62-77): the envelope of the
    absolute deviations of the variants from the nominal value."""
    sigma = _zero_like(nominal_value)
    values, sigmas = [], []
    for v in variants:
        value, sigma_mc = evaluate(v)
        value, sigma_mc = _as_value(value), _as_value(sigma_mc)
        values.append(value)
        sigmas.append(sigma_mc)
        sigma = np.maximum(sigma, np.abs(value - nominal_value))
        if np.ndim(sigma) == 0:
            sigma = float(sigma)
    return SystematicSourceResult(sigma, nominal_value, values, sigmas, list(labels))


def _collect_threshold_variants(nominal, threshold_factors):
    """_collect_threshold_variants (src/Uncertainty.jl:79-103): the scaled
    thresholds that are positive, distinct from the nominal one
    (isapprox with atol eps, rtol sqrt(eps)) and from each other."""
    variants, labels = [], []
    t0 = float(nominal.energy_threshold_low)
    if t0 <= 0.0:
        return variants, labels
    eps = np.finfo(np.float64).eps
    seen = set()
    for f in threshold_factors:
        t = float(f) * t0
        if t <= 0.0:
            continue
        if abs(t - t0) <= max(eps, math.sqrt(eps) * max(abs(t), abs(t0))):
            continue
        if t in seen:
            continue
        seen.add(t)
        variants.append(TransportVariation(nominal.straggling, nominal.scattering, t,
                                           nominal.seed))
        labels.append(f"threshold={t!r}")
    return variants, labels


def estimate_transport_uncertainty(evaluate, *, straggling=True, scattering=True,
                                   energy_threshold_low=100.0, seed=42,
                                   threshold_factors=(0.5, 2.0)):
    """estimate_transport_uncertainty (src/Uncertainty.jl:111-169).

    evaluate(TransportVariation) returns (value, sigma_mc), scalars or
    arrays of one shape.  Sources: "straggling", "scattering" (each toggled
    once) and "energy_threshold_low" (the nominal threshold times each
    factor); sigma_syst = sqrt(sum of the squared source envelopes),
    sigma_total = sqrt(sigma_mc^2 + sigma_syst^2)."""
    nominal = TransportVariation(bool(straggling), bool(scattering),
                                 float(energy_threshold_low), int(seed))
    value, sigma_mc = evaluate(nominal)
    value, sigma_mc = _as_value(value), _as_value(sigma_mc)
    sources = {}
    sources["straggling"] = _evaluate_source(
        evaluate, value,
        [TransportVariation(not nominal.straggling, nominal.scattering,
                            nominal.energy_threshold_low, nominal.seed)],
        [f"straggling={str(not nominal.straggling).lower()}"])
    sources["scattering"] = _evaluate_source(
        evaluate, value,
        [TransportVariation(nominal.straggling, not nominal.scattering,
                            nominal.energy_threshold_low, nominal.seed)],
        [f"scattering={str(not nominal.scattering).lower()}"])
    tv, tl = _collect_threshold_variants(nominal, threshold_factors)
    sources["energy_threshold_low"] = _evaluate_source(evaluate, value, tv, tl)
    syst = _zero_like(value)
    for s in sources.values():
        syst = syst + np.square(s.sigma)
    syst = np.sqrt(syst)
    total = np.sqrt(np.square(sigma_mc) + np.square(syst))
    if np.ndim(value) == 0:
        syst, total = float(syst), float(total)
    return TransportUncertaintyResult(value, sigma_mc, syst, total, sources, nominal)


def compute_flux_uncertainty(physics, rock_density, rock_thickness, elevation, energy_min,
                             energy_max, *, n_samples=1000, seed=42, straggling=True,
                             scattering=True, energy_threshold_low=100.0,
                             threshold_factors=(0.5, 2.0), porous_material=-1,
                             porous_density=0.0, porous_thickness=0.0,
                             primary_altitude=PRIMARY_ALTITUDE, precision="fp64"):
    """compute_flux_uncertainty (src/Uncertainty.jl:178-222): the budget of
    compute_flux on the device, every variation on the nominal seed."""
    from . import compute_flux

    def evaluate(v):
        return compute_flux(physics, rock_density, rock_thickness, elevation, energy_min,
                            energy_max, n_samples=n_samples, seed=v.seed,
                            straggling=v.straggling, scattering=v.scattering,
                            energy_threshold_low=v.energy_threshold_low,
                            porous_material=porous_material, porous_density=porous_density,
                            porous_thickness=porous_thickness,
                            primary_altitude=primary_altitude, precision=precision)

    return estimate_transport_uncertainty(evaluate, straggling=straggling, scattering=scattering,
                                          energy_threshold_low=energy_threshold_low, seed=seed,
                                          threshold_factors=threshold_factors)


def relative_uncertainty_percent(value, sigma, floor=1e-30):
    """relative_uncertainty_percent (src/Uncertainty.jl:230-237)."""
    d = np.maximum(np.abs(np.asarray(value, np.float64)), floor)
    r = 100.0 * np.asarray(sigma, np.float64) / d
    return float(r) if np.ndim(r) == 0 else r

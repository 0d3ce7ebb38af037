"""CSDA -> MC correction calibration over the device water-fraction CSDA model.

calibrate_csda_correction (src/Tomography.jl:1043-1179) fits the hard-loss
coefficient kappa_hard by a coarse-to-fine 1-D grid and then the geometric
residual by ridged least squares; calibrate_csda_material_correction
(src/Tomography_material_calibration.jl:1-61) fits the two material
coefficients to paired log-flux contrasts; save_csda_corrections /
load_csda_corrections (:63-92) keep both corrections in a TOML artifact.

The reference evaluates compute_directional_flux_csda bin by bin for every
trial coefficient.  Here the calibration bins form one CsdaBatch (paths and
energy samples resident on the device) and every objective evaluation is one
dp_dir_csda launch over all bins (the water fractions go up, the fluxes come
back); the corrections in force are read at each launch, as the reference
reads them at each evaluation.
"""
import json
import math
import numbers

import numpy as np

from .directional import (CsdaBatch, cell_density, get_csda_correction,
                          get_csda_material_correction, set_csda_correction,
                          set_csda_material_correction)
from . import directional as _dir


def path_rock_length(path):
    """Geometric rock path length (m): cells plus the rock remainder
    (src/Tomography.jl:394-400)."""
    L = path.remaining_rock_distance
    for s in path.segments:
        L += s.distance
    return L


def csda_geom_multiplier(path):
    """exp(a + b logL + c logL^2 + d cos zenith) of the installed correction,
    1 when no residual coefficient is set (src/Tomography.jl:405-412)."""
    c = get_csda_correction()
    if not (c.enabled and (c.resid_a != 0.0 or c.resid_b != 0.0 or c.resid_c != 0.0 or
                           c.resid_d != 0.0)):
        return 1.0
    logL = math.log(max(path_rock_length(path), 1.0))
    cos_t = math.cos(math.radians(path.zenith))
    return math.exp(c.resid_a + c.resid_b * logL + c.resid_c * logL * logL + c.resid_d * cos_t)


def column_water_fraction(matcfg, path, shallow_flags, water_fractions):
    """Water mass fraction of the whole rock column, dry remainder included
    (_column_water_fraction, src/Tomography.jl:560-570)."""
    water = 0.0
    mass = path.remaining_rock_distance * matcfg.rock_density
    for s in path.segments:
        wk = float(water_fractions[s.cell_idx - 1])
        gx = s.distance * cell_density(wk, bool(shallow_flags[s.cell_idx - 1]), matcfg)
        water += wk * gx
        mass += gx
    return water / max(mass, 1e-30)


def csda_material_multiplier(path, shallow_flags, matcfg, water_fractions):
    """exp(linear q + quadratic q^2) of the installed material correction
    (src/Tomography.jl:571-580)."""
    q = column_water_fraction(matcfg, path, shallow_flags, water_fractions)
    c = get_csda_material_correction()
    return math.exp(c.linear * q + c.quadratic * q * q) if c.enabled else 1.0


def _bin_model(physics, shallow_flags, matcfg, site, paths, bins, energy_samples, model):
    if model is not None:
        return model
    return CsdaBatch(physics, shallow_flags, matcfg, site, [paths[b - 1] for b in bins],
                     energy_samples).to_device()


def _fluxes(model, w, precision):
    return np.asarray(model.run(w, jacobian=False, precision=precision)[0], np.float64)


def calibrate_csda_correction(physics, shallow_flags, matcfg, site, paths, water_fractions,
                              energy_samples, mc_fluxes, bin_indices, *,
                              kh_grid=None, refine=4, fit_geometric=True, alpha_strag=1.0,
                              kh_anchor=None, kh_anchor_weight=0.0, ridge_geom=1e-3,
                              precision="fp64", model=None):
    """calibrate_csda_correction (src/Tomography.jl:1061-1179).

    bin_indices are 1-based indices into paths; mc_fluxes[i] is the MC flux of
    bin bin_indices[i].  Minimises mean(log(flux_csda / flux_mc)^2) (+ the
    optional ridge toward kh_anchor) over kappa_hard by a coarse-to-fine grid
    (kh_grid, default 0..80 in 41 points, then `refine` rounds of 9 points
    around the best), with alpha_strag pinned; with fit_geometric, fits the
    residual exp(a + b logL + c logL^2 + d cos zenith) by ridged least
    squares, else keeps the installed one.  Installs the result and returns
    (alpha_strag, kappa_hard, stats).  `model` replaces the device batch of
    the calibration bins (anything with CsdaBatch.run)."""
    mc_fluxes = np.asarray(mc_fluxes, np.float64)
    bin_indices = [int(b) for b in bin_indices]
    if len(mc_fluxes) != len(bin_indices):
        raise ValueError("mc_fluxes and bin_indices differ in length")
    valid = [i for i in range(len(bin_indices))
             if math.isfinite(mc_fluxes[i]) and mc_fluxes[i] > 0]
    if not valid:
        raise RuntimeError("calibrate_csda_correction: no positive MC reference fluxes")
    logmc = [math.log(mc_fluxes[i]) for i in valid]
    bins = [bin_indices[i] for i in valid]
    model = _bin_model(physics, shallow_flags, matcfg, site, paths, bins, energy_samples, model)
    w = np.ascontiguousarray(water_fractions, np.float64)

    cur = get_csda_correction()
    fa, fb, fc, fd = ((0.0, 0.0, 0.0, 0.0) if fit_geometric
                      else (cur.resid_a, cur.resid_b, cur.resid_c, cur.resid_d))

    def set_corr(kh):
        set_csda_correction(enabled=True, kappa_strag=alpha_strag, kappa_hard=kh, resid_a=fa,
                            resid_b=fb, resid_c=fc, resid_d=fd)

    def anchor_pen(kh):
        if kh_anchor is None or kh_anchor_weight <= 0.0:
            return 0.0
        return kh_anchor_weight * (kh - kh_anchor) ** 2

    def objective(kh):
        set_corr(kh)
        f = _fluxes(model, w, precision)
        s, n = 0.0, 0
        for j in range(len(bins)):
            if not (math.isfinite(f[j]) and f[j] > 0):
                continue
            d = math.log(f[j]) - logmc[j]
            s += d * d
            n += 1
        return math.inf if n == 0 else s / n + anchor_pen(kh)

    def rel_only():
        f = _fluxes(model, w, precision)
        acc, n = 0.0, 0
        for j in range(len(bins)):
            if not (math.isfinite(f[j]) and f[j] > 0):
                continue
            acc += abs(1.0 - f[j] / math.exp(logmc[j]))
            n += 1
        return math.nan if n == 0 else acc / n

    # "before": pure CSDA (no straggling enhancement, no hard-loss deficit)
    set_csda_correction(enabled=True, kappa_strag=0.0, kappa_hard=0.0, resid_a=fa, resid_b=fb,
                        resid_c=fc, resid_d=fd)
    rel_before = rel_only()

    best_kh, best_obj = 0.0, math.inf
    khg = [float(x) for x in (np.linspace(0.0, 80.0, 41) if kh_grid is None else kh_grid)]
    for _ in range(refine + 1):
        for kh in khg:
            o = objective(kh)
            if o < best_obj:
                best_obj, best_kh = o, kh
        dkh = khg[1] - khg[0] if len(khg) > 1 else 0.5
        khg = [float(x) for x in np.linspace(max(0.0, best_kh - dkh), best_kh + dkh, 9)]
    best_ks = alpha_strag

    ra, rb, rc, rd = fa, fb, fc, fd
    if fit_geometric:
        set_csda_correction(enabled=True, kappa_strag=best_ks, kappa_hard=best_kh)
        f = _fluxes(model, w, precision)
        feats, ys = [], []
        for j, b in enumerate(bins):
            if not (math.isfinite(f[j]) and f[j] > 0):
                continue
            p = paths[b - 1]
            logL = math.log(max(path_rock_length(p), 1.0))
            feats.append([1.0, logL, logL * logL, math.cos(math.radians(p.zenith))])
            ys.append(logmc[j] - math.log(f[j]))
        ra = rb = rc = rd = 0.0
        if len(ys) >= 4:
            A = np.array(feats)
            R = np.diag([0.0, ridge_geom, ridge_geom, ridge_geom])
            ra, rb, rc, rd = (float(v) for v in np.linalg.solve(A.T @ A + R, A.T @ np.array(ys)))
        elif ys:
            ra = sum(ys) / len(ys)

    set_csda_correction(enabled=True, kappa_strag=best_ks, kappa_hard=best_kh, resid_a=ra,
                        resid_b=rb, resid_c=rc, resid_d=rd)
    rel_after = rel_only()
    stats = dict(rel_before=rel_before, rel_after=rel_after, mse_log=best_obj,
                 n_bins=len(bins), kappa_strag=best_ks, kappa_hard=best_kh, resid_a=ra,
                 resid_b=rb, resid_c=rc, resid_d=rd)
    return best_ks, best_kh, stats


def calibrate_csda_material_correction(physics, shallow_flags, matcfg, site, paths, baseline,
                                       fields, energy_samples, mc_baseline, mc_fields, bins, *,
                                       ridge=1e-6, precision="fp64", model=None):
    """calibrate_csda_material_correction
    (src/Tomography_material_calibration.jl:14-61).

    mc_fields[j][k] is the MC flux of field j in bin bins[k] (1-based path
    indices), mc_baseline[k] that of the baseline field.  With the material
    correction off, every (bin, field) pair gives the row (q - q0, q^2 - q0^2)
    and the target log(m / m0) - log(f / f0); (linear, quadratic) solve the
    ridged normal equations and are installed.  On any error the previous
    material correction is restored."""
    fields = [np.ascontiguousarray(f, np.float64) for f in fields]
    bins = [int(b) for b in bins]
    if len(fields) < 2:
        raise ValueError("at least two material training fields required")
    mc_fields = np.asarray(mc_fields, np.float64)
    if mc_fields.shape != (len(fields), len(bins)):
        raise ValueError("MC field/bin matrix")
    mc_baseline = np.asarray(mc_baseline, np.float64)
    if len(mc_baseline) != len(bins):
        raise ValueError("MC baseline")
    if not (ridge >= 0 and math.isfinite(ridge)):
        raise ValueError("invalid ridge")
    baseline = np.ascontiguousarray(baseline, np.float64)
    for w in (baseline, *fields):
        if len(w) != len(shallow_flags):
            raise ValueError("field length")
        if not np.all(np.isfinite(w) & (w >= 0) & (w <= 1)):
            raise ValueError("mass fractions outside [0,1]")
    old = get_csda_material_correction()
    try:
        set_csda_material_correction(enabled=False)
        model = _bin_model(physics, shallow_flags, matcfg, site, paths, bins, energy_samples,
                           model)
        f0s = _fluxes(model, baseline, precision)
        fs = [_fluxes(model, w, precision) for w in fields]
        rows, targets, qs = [], [], []
        for k, b in enumerate(bins):
            path = paths[b - 1]
            f0, m0 = f0s[k], mc_baseline[k]
            if not (math.isfinite(f0) and f0 > 0 and math.isfinite(m0) and m0 > 0):
                raise ValueError("invalid baseline flux")
            q0 = column_water_fraction(matcfg, path, shallow_flags, baseline)
            for j, w in enumerate(fields):
                f, m = fs[j][k], mc_fields[j, k]
                if not (math.isfinite(f) and f > 0 and math.isfinite(m) and m > 0):
                    raise ValueError("invalid training flux")
                q = column_water_fraction(matcfg, path, shallow_flags, w)
                rows.append([q - q0, q * q - q0 * q0])
                qs.append(q)
                targets.append(math.log(m / m0) - math.log(f / f0))
        A = np.array(rows)
        t = np.array(targets)
        if np.linalg.matrix_rank(A) != 2:
            raise ValueError("material training contrasts do not identify two coefficients")
        coef = np.linalg.solve(A.T @ A + ridge * np.eye(2), A.T @ t)
        prediction = A @ coef
        set_csda_material_correction(linear=float(coef[0]), quadratic=float(coef[1]))
        return dict(linear=float(coef[0]), quadratic=float(coef[1]), ridge=float(ridge),
                    condition_number=float(np.linalg.cond(A)), q_min=min(qs), q_max=max(qs),
                    n_fields=len(fields), bins=list(bins), n_pairs=len(targets),
                    rms_log_before=math.sqrt(float(np.sum(t * t)) / len(t)),
                    rms_log_after=math.sqrt(float(np.sum((prediction - t) ** 2)) / len(t)),
                    baseline=baseline.tolist(), training_fields=[w.tolist() for w in fields])
    except BaseException:
        _dir._MATERIAL_CORRECTION = old
        raise


# ------------------------------------------------------------ correction artifact
_CSDA_KEYS = ("kappa_strag", "kappa_hard", "resid_a", "resid_b", "resid_c", "resid_d")


def _toml_value(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, numbers.Integral):
        return str(int(v))
    if isinstance(v, numbers.Real):
        x = float(v)
        if math.isnan(x):
            return "nan"
        if math.isinf(x):
            return "inf" if x > 0 else "-inf"
        return repr(x)
    if isinstance(v, str):
        return json.dumps(v)
    if isinstance(v, (list, tuple, np.ndarray)):
        return "[" + ", ".join(_toml_value(x) for x in v) + "]"
    raise TypeError(f"metadata value of type {type(v).__name__} has no TOML form")


def save_csda_corrections(path, metadata=None):
    """save_csda_corrections (src/Tomography_material_calibration.jl:63-74):
    the installed dry and material corrections with user provenance, schema
    version 1, as TOML."""
    base, material = get_csda_correction(), get_csda_material_correction()
    lines = ["schema_version = 1", "", "[csda]", f"enabled = {_toml_value(base.enabled)}"]
    lines += [f"{k} = {_toml_value(getattr(base, k))}" for k in _CSDA_KEYS]
    lines += ["", "[material]", f"enabled = {_toml_value(material.enabled)}",
              f"linear = {_toml_value(material.linear)}",
              f"quadratic = {_toml_value(material.quadratic)}", "", "[metadata]"]
    for k, v in (metadata or {}).items():
        lines.append(f"{json.dumps(str(k))} = {_toml_value(v)}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def load_csda_corrections(path):
    """load_csda_corrections! (src/Tomography_material_calibration.jl:76-92):
    validates every field of a version-1 artifact, then installs both
    corrections at once; returns the metadata."""
    import tomllib
    with open(path, "rb") as f:
        data = tomllib.load(f)
    if data.get("schema_version") != 1:
        raise ValueError("unsupported correction schema")
    b, m = data["csda"], data["material"]
    if not (isinstance(b["enabled"], bool) and isinstance(m["enabled"], bool)):
        raise ValueError("enabled must be Boolean")
    bv = [float(b[k]) for k in _CSDA_KEYS]
    mv = [float(m[k]) for k in ("linear", "quadratic")]
    if not all(math.isfinite(x) for x in bv + mv):
        raise ValueError("nonfinite correction coefficients")
    _dir._CORRECTION = _dir.CsdaCorrection(b["enabled"], *bv)
    _dir._MATERIAL_CORRECTION = _dir.CsdaMaterialCorrection(m["enabled"], *mv)
    return data.get("metadata", {})

"""Water-fraction CSDA model on the GPU (compute_directional_flux_csda,
directional_flux_and_grad_csda, assemble_forward_and_jacobian,
src/Tomography.jl:444-820) against the oracle, through the C ABI: flux and
d flux / d w in FP64 (and the mixed-precision walk within 1e-4), with the
corrections off and on."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CFG0 = [0, 2, 1, -1]


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


@pytest.fixture(scope="module")
def orc_phys(oracle):
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), n=80,
                                  Kmin=1e-3, Kmax=1e6)


@pytest.fixture(scope="module")
def phys(dp, orc_phys):
    return dp.upload_physics([orc_phys.table(i) for i in range(3)], ["StandardRock", "Air", "Water"])


@pytest.fixture(scope="module")
def scene(dp):
    """48 cells; the reference's two test paths and 62 seeded paths of 1-14
    segments (some crossing a cell twice), rock beyond the cells, site
    (963, 30000)."""
    rng = np.random.default_rng(11)
    n_cells = 48
    wf = rng.uniform(0.0, 0.4, n_cells)
    paths = [
        dp.DirectionalPath(20.0, 0.0, [dp.CellSegment(1, 30.0), dp.CellSegment(2, 40.0),
                                       dp.CellSegment(3, 30.0)], 100.0, 100.0, 0.0, 60.0, True),
        dp.DirectionalPath(35.0, 90.0, [dp.CellSegment(2, 50.0), dp.CellSegment(4, 35.0)],
                           85.0, 85.0, 0.0, 55.0, True)]
    for _ in range(62):
        k = int(rng.integers(1, 15))
        cells = rng.integers(1, n_cells + 1, k)
        segs = [dp.CellSegment(int(c), float(rng.uniform(2.0, 40.0))) for c in cells]
        paths.append(dp.DirectionalPath(float(rng.uniform(0.0, 70.0)), 0.0, segs, 0.0, 0.0,
                                        float(rng.uniform(0.0, 300.0)),
                                        float(rng.uniform(40.0, 400.0)), True))
    return wf, paths


def _samples(dp, n, seed):
    rng = np.random.default_rng(seed)
    rk = math.log(1e6 / 1e-3)
    E = 1e-3 * np.exp(rk * rng.random(n))
    q = np.where(rng.random(n) > 0.5, 1.0, -1.0)
    return [dp.EnergySample(e, c, e * rk) for e, c in zip(E, q)]


def _oracle(oracle, orc_phys, wf, paths, samples, corr, shallow=None, cfg=CFG0,
            dens=(2650.0, 1000.0, 0.0, 0.0)):
    seg_ptr = np.concatenate([[0], np.cumsum([len(p.segments) for p in paths])])
    cells = [s.cell_idx - 1 for p in paths for s in p.segments]
    lens = [s.distance for p in paths for s in p.segments]
    return oracle.dir_csda(orc_phys, cfg, list(dens), [963.0, 3e4], corr,
                           [math.cos(math.radians(p.zenith)) for p in paths],
                           [p.remaining_rock_distance for p in paths],
                           [p.surface_exit_z for p in paths], [int(p.valid) for p in paths],
                           seg_ptr, cells, lens,
                           np.zeros(len(wf), np.uint8) if shallow is None else shallow, wf,
                           [s.energy for s in samples], [s.charge for s in samples],
                           [s.weight for s in samples], grad=True)


def _per_cell_first(seg_ptr, cells, jac):
    """Device per-segment values summed per cell, at the cell's first segment."""
    out = np.zeros(len(jac))
    for b in range(len(seg_ptr) - 1):
        first = {}
        for k in range(seg_ptr[b], seg_ptr[b + 1]):
            c = cells[k]
            if c not in first:
                first[c] = k
            out[first[c]] += jac[k]
    return out


CORR = {"plain": None,
        "correction": dict(enabled=True, kappa_strag=1.0, kappa_hard=7.0, resid_a=0.1,
                           resid_b=-0.05, resid_c=0.01, resid_d=0.2),
        "material": "material"}


@pytest.mark.parametrize("which", list(CORR))
def test_flux_and_jacobian_match_oracle(dp, phys, oracle, orc_phys, scene, which):
    wf, paths = scene
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    samples = _samples(dp, 24, 5)
    corr = [0] * 10
    try:
        if which == "correction":
            dp.set_csda_correction(**CORR[which])
            c = CORR[which]
            corr = [1, c["kappa_strag"], c["kappa_hard"], c["resid_a"], c["resid_b"], c["resid_c"],
                    c["resid_d"], 0, 0.0, 0.0]
        elif which == "material":
            dp.set_csda_material_correction(enabled=True, linear=0.4, quadratic=-0.3)
            corr = [0] * 7 + [1, 0.4, -0.3]
        f, seg_ptr, cells, jac = dp.csda_flux_batch(phys, np.zeros(len(wf), bool), cfg, site, paths,
                                                    wf, samples)
    finally:
        dp.set_csda_correction(enabled=False)
        dp.set_csda_material_correction(enabled=False)
    of, og = _oracle(oracle, orc_phys, wf, paths, samples, corr)
    assert np.all(np.isfinite(f)) and np.all(f > 0)
    np.testing.assert_allclose(f, of, rtol=1e-10, atol=0)
    g = _per_cell_first(seg_ptr, cells, jac)
    np.testing.assert_allclose(g, og, rtol=1e-8, atol=1e-12 * np.abs(og).max())


def test_porous_top_layer(dp, phys, oracle, orc_phys, scene):
    """Shallow cells with a porous top layer (the porous/rock/water mixture of
    src/Tomography.jl:303-352); the porous material here is rock at 1800 kg/m^3."""
    wf, paths = scene
    cfg = dp.MaterialConfig(1, 3, 2, 1, 2650.0, 1000.0, 1800.0, 20.0)
    site = dp.SiteConfig(963.0, 3e4)
    samples = _samples(dp, 16, 6)
    shallow = (np.arange(len(wf)) % 2 == 0)
    f, seg_ptr, cells, jac = dp.csda_flux_batch(phys, shallow, cfg, site, paths, wf, samples)
    of, og = _oracle(oracle, orc_phys, wf, paths, samples, [0] * 10,
                     shallow=shallow.astype(np.uint8), cfg=[0, 2, 1, 0],
                     dens=(2650.0, 1000.0, 1800.0, 20.0))
    np.testing.assert_allclose(f, of, rtol=1e-10, atol=0)
    np.testing.assert_allclose(_per_cell_first(seg_ptr, cells, jac), og, rtol=1e-8,
                               atol=1e-12 * np.abs(og).max())


def test_jacobian_vs_finite_differences(dp, phys, scene):
    """The device Jacobian against central FD of the device flux
    (test/test_tomography.jl:101-116, rtol 1e-4)."""
    wf, paths = scene
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    samples = _samples(dp, 8, 7)
    sh = np.zeros(len(wf), bool)
    flux, ids, vals = dp.directional_flux_and_grad_csda(phys, sh, cfg, site, paths[0], wf, samples)
    h = 1e-5
    for c, v in zip(ids, vals):
        wp, wm = wf.copy(), wf.copy()
        wp[c - 1] += h
        wm[c - 1] -= h
        fd = (dp.compute_directional_flux_csda(phys, sh, cfg, site, paths[0], wp, samples) -
              dp.compute_directional_flux_csda(phys, sh, cfg, site, paths[0], wm, samples)) / (2 * h)
        assert v == pytest.approx(fd, rel=1e-4)


def test_assembled_jacobian_and_invalid_paths(dp, phys, scene):
    """assemble_forward_and_jacobian: one row per bin, on-path cells only, the
    per-bin gradients; an invalid path gives NaN and an empty row."""
    wf, paths = scene
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    samples = _samples(dp, 8, 8)
    sh = np.zeros(len(wf), bool)
    ps = list(paths[:6]) + [paths[6]._replace(valid=False)]
    flux, J = dp.assemble_forward_and_jacobian(phys, sh, cfg, site, ps, wf, samples,
                                               n_cells=len(wf))
    assert J.shape == (7, len(wf))
    assert np.isnan(flux[6]) and J.getrow(6).nnz == 0
    for b in range(6):
        f, ids, vals = dp.directional_flux_and_grad_csda(phys, sh, cfg, site, ps[b], wf, samples)
        assert f == flux[b]
        row = J.getrow(b).toarray().ravel()
        assert set(np.nonzero(row)[0] + 1) <= set(ids)
        np.testing.assert_allclose(row[np.array(ids) - 1], vals, rtol=1e-12, atol=0)


@pytest.mark.parametrize("which", ["plain", "correction"])
def test_mixed_precision_within_1e4(dp, phys, oracle, orc_phys, scene, which):
    """FP32 walk and tangents (FP64 adjoint sums, flux and reductions): flux
    within 1e-4 of the FP64 oracle per direction, the Jacobian within 1e-4
    norm-wise per direction."""
    wf, paths = scene
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    samples = _samples(dp, 32, 9)
    corr = [0] * 10
    try:
        if which == "correction":
            dp.set_csda_correction(**CORR[which])
            c = CORR[which]
            corr = [1, c["kappa_strag"], c["kappa_hard"], c["resid_a"], c["resid_b"], c["resid_c"],
                    c["resid_d"], 0, 0.0, 0.0]
        f, seg_ptr, cells, jac = dp.csda_flux_batch(phys, np.zeros(len(wf), bool), cfg, site, paths,
                                                    wf, samples, precision="mixed")
    finally:
        dp.set_csda_correction(enabled=False)
    of, og = _oracle(oracle, orc_phys, wf, paths, samples, corr)
    np.testing.assert_allclose(f, of, rtol=1e-4, atol=0)
    g = _per_cell_first(seg_ptr, cells, jac)
    worst = 0.0
    for b in range(len(paths)):
        a, z = seg_ptr[b], seg_ptr[b + 1]
        if z > a:
            worst = max(worst, np.linalg.norm(g[a:z] - og[a:z]) / np.linalg.norm(og[a:z]))
    print("mixed-precision Jacobian, worst per-direction relative norm error", worst)
    assert worst <= 1e-4

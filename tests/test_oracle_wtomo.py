"""The oracle's water-fraction CSDA model (compute_directional_flux_csda and
its gradient, src/Tomography.jl:444-820) against the reference's own checks
(test/test_tomography.jl:19-121): central finite differences with the
corrections off and on, and the charge-0 quadrature identity (CPU only)."""
import math

import numpy as np
import pytest

# test/test_tomography.jl:19-44: two paths over four cells, site (1000, 12000)
CFG = [0, 2, 1, -1]                 # rock, water, air, no porous (0-based)
DENS = [2650.0, 1000.0, 0.0, 0.0]
SITE = [1000.0, 12000.0]
WF = np.array([0.10, 0.20, 0.05, 0.15])
PATHS = [  # cos(zenith), remaining rock, surface exit z, (cell, length) segments
    (math.cos(math.radians(20.0)), 0.0, 60.0, [(0, 30.0), (1, 40.0), (2, 30.0)]),
    (math.cos(math.radians(35.0)), 0.0, 55.0, [(1, 50.0), (3, 35.0)]),
]
OFF = [0] * 10
ON = [1, 1.0, 7.0, 0.1, -0.05, 0.01, 0.2, 0, 0.0, 0.0]  # :120-121 settings
MAT = [0] * 7 + [1, 0.4, -0.3]


@pytest.fixture(scope="module")
def phys(oracle):
    """create_physics(MUON; n_energies=80, K_min=1e-3, K_max=1e6, [rock, air, water])."""
    return oracle.default_physics((oracle.STANDARD_ROCK, oracle.AIR, oracle.WATER), n=80,
                                  Kmin=1e-3, Kmax=1e6)


def _samples(n, seed):
    rng = np.random.default_rng(seed)
    rk = math.log(1e6 / 1e-3)
    E = 1e-3 * np.exp(rk * rng.random(n))
    return E, np.where(rng.random(n) > 0.5, 1.0, -1.0), E * rk


def _run(oracle, phys, corr, wf, E, q, w, grad=False, paths=PATHS):
    seg_ptr = np.concatenate([[0], np.cumsum([len(p[3]) for p in paths])])
    cells = [c for p in paths for c, _ in p[3]]
    lens = [l for p in paths for _, l in p[3]]
    return oracle.dir_csda(phys, CFG, DENS, SITE, corr, [p[0] for p in paths],
                           [p[1] for p in paths], [p[2] for p in paths], [1] * len(paths),
                           seg_ptr, cells, lens, np.zeros(len(wf), np.uint8), wf, E, q, w,
                           grad=grad)


@pytest.mark.parametrize("corr", [OFF, ON, MAT], ids=["plain", "correction", "material"])
def test_gradient_matches_finite_differences(oracle, phys, corr):
    """test/test_tomography.jl:97-137: d flux / d w against central FD (the
    reference's rtol 1e-4)."""
    E, q, w = _samples(6, 42)
    f, g = _run(oracle, phys, corr, WF, E, q, w, grad=True)
    assert np.all(np.isfinite(f)) and np.all(f > 0)
    h = 1e-5
    k = 0
    for b, p in enumerate(PATHS):
        for c, _ in p[3]:
            wp, wm = WF.copy(), WF.copy()
            wp[c] += h
            wm[c] -= h
            fd = (_run(oracle, phys, corr, wp, E, q, w)[b] -
                  _run(oracle, phys, corr, wm, E, q, w)[b]) / (2 * h)
            assert g[k] == pytest.approx(fd, rel=1e-4), (b, c)
            k += 1


def test_charge_zero_nodes_equal_paired_charges(oracle, phys):
    """test/test_tomography.jl:71-80: a charge-0 quadrature node equals the
    average of explicit +-1 charges with twice its weight (to 1e-13)."""
    import dpgpu
    E, q, w = dpgpu.csda_energy_quadrature(32, 1.0, 100.0)
    Ep = np.repeat(E, 2)
    qp = np.tile([-1.0, 1.0], len(E))
    wp = np.repeat(2 * w, 2)
    a = _run(oracle, phys, OFF, WF, E, q, w)
    b = _run(oracle, phys, OFF, WF, Ep, qp, wp)
    np.testing.assert_allclose(a, b, rtol=1e-13)


def test_invalid_path_is_nan(oracle, phys):
    """src/Tomography.jl:676-678: an invalid path (or cos zenith <= 0) gives NaN."""
    E, q, w = _samples(4, 1)
    bad = [(-0.2, 0.0, 10.0, [(0, 10.0)])]
    assert np.isnan(_run(oracle, phys, OFF, WF, E, q, w, paths=bad)[0])

"""Paths traced through real-geometry volumes (a terrain surface over a
tetrahedral mesh, examples/lvd_tomography.jl:694-736, 835-861, and a voxel
volume under the same terrain) feed the device kernels: the water-fraction
CSDA model with its Jacobian (dp_dir_csda) and the fixed-path stochastic MC
(dp_dir_mc).  Each is compared with the oracle run on the oracle's own
traced paths (oracle/topo_paths.py), so the test covers the tracing and the
device transport together."""
import math

import numpy as np
import pytest

from test_gpu_dir import _oracle_batch
from test_gpu_mc import _agree
from test_gpu_wtomo import _oracle as _oracle_csda
from test_gpu_wtomo import _per_cell_first
from test_topography import EDGES, T, _kuhn_mesh, _terrains

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
    return dp.upload_physics([orc_phys.table(i) for i in range(3)], ["StandardRock", "Air", "Water"],
                             materials=(dp.STANDARD_ROCK, dp.AIR, dp.WATER))


@pytest.fixture(scope="module")
def traced(dp):
    """Library and oracle traces of 12 directions through the Kuhn mesh
    (1536 tetrahedra of the 8 x 8 x 4 box grid) under the synthetic terrain."""
    t, ot = _terrains(dp)
    pts, tets, _ = _kuhn_mesh(*EDGES)
    vol = dp.TetraVolume(pts, tets)
    nb = T.tetra_neighbors(tets)
    zen, az = [15.0, 35.0, 50.0], [20.0, 110.0, 200.0, 290.0]
    lib_paths = dp.precompute_paths(vol, zen, az, t)
    orc_paths = []
    for z in zen:
        for a in az:
            segs, tr, S, rem, ez, ok = T.trace_tetra(pts, tets, nb, ot, z, a)
            orc_paths.append(dp.DirectionalPath(z, a, [dp.CellSegment(int(c), float(l))
                                                       for c, l in segs],
                                                tr, S, rem, ez, ok))
    assert all(p.valid for p in lib_paths) and len(lib_paths) == 12
    for a, b in zip(lib_paths, orc_paths):
        assert [s.cell_idx for s in a.segments] == [s.cell_idx for s in b.segments]
    return len(tets), lib_paths, orc_paths


def test_tetra_paths_through_csda_model(dp, phys, oracle, orc_phys, traced):
    """compute_directional_flux_csda / directional_flux_and_grad_csda over the
    library's tetrahedral paths (FP64) against the oracle over its own paths:
    flux to 1e-9 and d flux / d w per cell to 1e-7 (the traces agree to
    1e-12 per segment)."""
    n_cells, lib_paths, orc_paths = traced
    wf = np.random.default_rng(12).uniform(0.0, 0.4, n_cells)
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    rng = np.random.default_rng(13)
    rk = math.log(1e6 / 1e-3)
    E = 1e-3 * np.exp(rk * rng.random(24))
    samples = [dp.EnergySample(e, c, e * rk)
               for e, c in zip(E, np.where(rng.random(24) > 0.5, 1.0, -1.0))]
    f, seg_ptr, cells, jac = dp.csda_flux_batch(phys, np.zeros(n_cells, bool), cfg, site,
                                                lib_paths, wf, samples)
    of, og = _oracle_csda(oracle, orc_phys, wf, orc_paths, samples, [0] * 10)
    assert np.all(f > 0)
    np.testing.assert_allclose(f, of, rtol=1e-9, atol=0)
    g = _per_cell_first(seg_ptr, cells, jac)
    np.testing.assert_allclose(g, og, rtol=1e-7, atol=1e-12 * np.abs(og).max())


def test_tetra_paths_through_fixed_path_mc(dp, phys, oracle, orc_phys, traced):
    """compute_directional_flux_mc over the library's tetrahedral paths
    (cells of rock or rock with 30 % water, straggling, FP64) against the
    oracle's histories on its own paths and the same streams: at least 99 %
    of the histories agree to 1e-9 and the paired differences average to
    zero within 3 of their standard errors."""
    n_cells, lib_paths, orc_paths = traced
    wf = np.where(np.arange(n_cells) % 4 == 1, 0.3, 0.0)
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2710.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    mats, dens = dp.build_cell_properties_for_mc(phys, np.zeros(n_cells, bool), wf, cfg)
    rng = np.random.default_rng(14)
    n_per = [300] * len(lib_paths)
    rk = math.log(1e5 / 0.5)
    samples = []
    for n in n_per:
        E = 0.5 * np.exp(rk * rng.random(n))
        q = np.where(rng.random(n) > 0.5, 1.0, -1.0)
        samples.append([(e, c, e * rk) for e, c in zip(E, q)])
    es = [[dp.EnergySample(*s) for s in ss] for ss in samples]
    r = dp.directional_flux_mc_batch(phys, cfg, site, lib_paths, mats, dens, es, 51,
                                     precision="fp64", return_histories=True)
    oc, ost, _, _ = _oracle_batch(dp, oracle, orc_phys, (cfg, site, mats, dens, orc_paths),
                                  samples, 51)
    assert np.all(ost == 0) and np.all(r["status"] == 0)
    assert _agree(r["contrib"], oc, 1e-9).mean() >= 0.99
    d = r["contrib"] - oc
    assert abs(d.mean()) <= 3 * d.std() / math.sqrt(len(d)) + 1e-14 * abs(oc.mean())
    assert (oc > 0).sum() > len(oc) // 10


def test_voxel_paths_under_terrain_through_csda_model(dp, phys, oracle, orc_phys):
    """The voxel march (trace_path(::VoxelVolume)) cut at the terrain's exit:
    the library's DirectionalPaths through the CSDA model against the oracle's
    restated march (oracle/voxel_paths.py) under the oracle's terrain."""
    import voxel_paths as V
    t, ot = _terrains(dp)
    vol = dp.VoxelVolume(*EDGES)
    zen, az = [10.0, 30.0, 45.0, 60.0], [0.0, 135.0, 250.0]
    lib_paths = dp.precompute_paths(vol, zen, az, t)
    orc_paths = []
    for z in zen:
        for a in az:
            S, ok, ez = ot.exit(T.direction_vector(z, a))
            assert ok
            cells, lens, tr = V.trace_path(EDGES, z, a, S)
            orc_paths.append(dp.DirectionalPath(z, a, [dp.CellSegment(int(c) + 1, float(l))
                                                       for c, l in zip(cells, lens)],
                                                tr, S, max(0.0, S - tr), ez, True))
    for p, q in zip(lib_paths, orc_paths):
        assert [s.cell_idx for s in p.segments] == [s.cell_idx for s in q.segments]
        np.testing.assert_allclose([s.distance for s in p.segments],
                                   [s.distance for s in q.segments], rtol=1e-12)
        assert p.remaining_rock_distance == pytest.approx(q.remaining_rock_distance, abs=1e-9)
    n_cells = (len(EDGES[0]) - 1) * (len(EDGES[1]) - 1) * (len(EDGES[2]) - 1)
    wf = np.random.default_rng(15).uniform(0.0, 0.4, n_cells)
    cfg = dp.MaterialConfig(1, 3, 2, -1, 2650.0, 1000.0, 0.0, 0.0)
    site = dp.SiteConfig(963.0, 3e4)
    rk = math.log(1e6 / 1e-3)
    rng = np.random.default_rng(16)
    E = 1e-3 * np.exp(rk * rng.random(16))
    samples = [dp.EnergySample(e, 0.0, e * rk) for e in E]
    f, seg_ptr, cells, jac = dp.csda_flux_batch(phys, np.zeros(n_cells, bool), cfg, site,
                                                lib_paths, wf, samples)
    of, og = _oracle_csda(oracle, orc_phys, wf, orc_paths, samples, [0] * 10)
    np.testing.assert_allclose(f, of, rtol=1e-9, atol=0)
    np.testing.assert_allclose(_per_cell_first(seg_ptr, cells, jac), og, rtol=1e-7,
                               atol=1e-12 * np.abs(og).max())

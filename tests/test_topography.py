"""Terrain and tetrahedral-mesh geometry (CPU): the elevation map and the
ray-triangle test against the reference's known answers
(test/runtests.jl:306-338, 389-399); the surface-exit search and the
tetrahedral walk against the oracle's restatement (oracle/topo_paths.py) on a
synthetic terrain and a Kuhn-subdivided box mesh; the tetrahedral paths
against the voxel march on the same box grid."""
import itertools
import math
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import topo_paths as T  # noqa: E402


@pytest.fixture(scope="module")
def dp():
    import dpgpu
    return dpgpu


def test_elevation_map_known_answers(dp):
    """test/runtests.jl:306-338: the plane z = x + 2y on an 11 x 11 map."""
    m = dp.ElevationMap(11, 11, (0.0, 10.0), (0.0, 10.0), (0.0, 100.0))
    for ix in range(11):
        for iy in range(11):
            m.fill(ix, iy, float(ix + 2 * iy))
    assert m.node(5, 3) == pytest.approx((5.0, 3.0, 11.0))
    z, inside = m.elevation(5.5, 3.5)
    assert inside[0] and z[0] == pytest.approx(12.5, abs=0.01)
    _, inside = m.elevation(-1.0, 5.0)
    assert not inside[0]
    gx, gy, gin = m.gradient(5.0, 5.0)
    assert gin[0] and gx[0] == pytest.approx(1.0, abs=0.2) and gy[0] == pytest.approx(2.0, abs=0.2)
    with pytest.raises(ValueError):
        m.fill(11, 0, 1.0)
    with pytest.raises(ValueError):
        dp.ElevationMap(4, 4, (0, 1), (0, 1), (5.0, 5.0))


def test_ray_triangle_known_answers(dp):
    """test/runtests.jl:389-399: a hit at distance 1 on z = 0, and a miss."""
    tri = ([0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0])
    hit, t, p = dp.ray_triangle_intersect([0.25, 0.25, 1.0], [0.0, 0.0, -1.0], *tri)
    assert hit and t == pytest.approx(1.0) and p[2] == pytest.approx(0.0)
    hit, _, _ = dp.ray_triangle_intersect([2.0, 2.0, 1.0], [0.0, 0.0, -1.0], *tri)
    assert not hit


DET = 963.0


def _terrain_data():
    """41 x 41 nodes over [-2, 2] km: a tilted, rippled surface 130-260 m
    above the detector."""
    xs = np.linspace(-2.0, 2.0, 41)
    X, Y = np.meshgrid(xs, xs)  # [iy][ix]
    return DET + 180.0 + 35.0 * np.sin(1.3 * X) * np.cos(0.9 * Y) + 12.0 * X


def _terrains(dp):
    data = _terrain_data()
    em = dp.ElevationMap(41, 41, (-2.0, 2.0), (-2.0, 2.0), (0.0, 2000.0), data=data)
    return (dp.Terrain(em, detector_elevation=DET),
            T.Terrain(41, 41, -2.0, -2.0, 0.1, 0.1, data, DET))


def _dirs(n, seed, zmax=80.0):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, zmax, n), rng.uniform(0.0, 360.0, n)


def test_surface_exit_matches_oracle(dp):
    """ray_surface_exit_distance for 200 directions (some leave the 2 km map
    or point down): the same distances and exit altitudes as the oracle."""
    t, ot = _terrains(dp)
    zen, az = _dirs(200, 1, zmax=95.0)
    d, z, ok = t.surface_exit(zen, az)
    assert 20 < ok.sum() < 200
    for i in range(200):
        s, o, e = ot.exit(T.direction_vector(zen[i], az[i]))
        assert bool(ok[i]) == o
        if o:
            assert d[i] == pytest.approx(s, rel=1e-14) and z[i] == pytest.approx(e, rel=1e-14)
    h = t.local_surface_height([0.0, 5000.0], [0.0, 0.0])
    assert h[0] == pytest.approx(ot.height(0.0, 0.0)) and math.isnan(h[1])


def _kuhn_mesh(x_edges, y_edges, z_edges):
    """Six tetrahedra per box along its main diagonal (a conforming mesh);
    points n x 3, tets m x 4 (1-based), and each tetrahedron's box."""
    nx, ny, nz = len(x_edges) - 1, len(y_edges) - 1, len(z_edges) - 1
    idx = {}
    pts = []
    for k, j, i in itertools.product(range(nz + 1), range(ny + 1), range(nx + 1)):
        idx[(i, j, k)] = len(pts) + 1
        pts.append((x_edges[i], y_edges[j], z_edges[k]))
    tets, box = [], []
    for k, j, i in itertools.product(range(nz), range(ny), range(nx)):
        for perm in itertools.permutations(range(3)):
            v = [0, 0, 0]
            chain = [idx[(i, j, k)]]
            for ax in perm:
                v[ax] += 1
                chain.append(idx[(i + v[0], j + v[1], k + v[2])])
            tets.append(chain)
            box.append(i + nx * (j + ny * k))
    return np.array(pts), np.array(tets, np.int32), np.array(box)


EDGES = (np.linspace(-301.3, 298.7, 9), np.linspace(-297.1, 302.9, 9), np.linspace(0.0, 300.0, 5))


def test_tetra_trace_matches_oracle(dp):
    """trace_path(::TetraVolume) on a 1536-tetrahedron mesh: the same
    tetrahedron sequence and segment lengths as the oracle, the same
    remaining rock and validity."""
    t, ot = _terrains(dp)
    pts, tets, _ = _kuhn_mesh(*EDGES)
    vol = dp.TetraVolume(pts, tets)
    nb = T.tetra_neighbors(tets)
    np.testing.assert_array_equal(vol.neighbors, nb)
    assert (vol.neighbors == 0).sum() == 2 * (8 * 8 * 2 + 8 * 4 * 2 + 8 * 4 * 2)  # boundary faces
    zen, az = _dirs(24, 2, zmax=75.0)
    zen = np.append(zen, [0.0, 100.0])
    az = np.append(az, [0.0, 30.0])
    seg_ptr, cells, lens, trav, dist, rem, ez, ok = dp.trace_tetra_paths(vol, t, zen, az)
    for i in range(len(zen)):
        segs, tr, S, r, e, o = T.trace_tetra(pts, tets, nb, ot, zen[i], az[i])
        assert bool(ok[i]) == o
        if not o:
            continue
        mine = list(zip(cells[seg_ptr[i]:seg_ptr[i + 1]], lens[seg_ptr[i]:seg_ptr[i + 1]]))
        assert [c for c, _ in mine] == [c for c, _ in segs]
        np.testing.assert_allclose([l for _, l in mine], [l for _, l in segs], rtol=1e-12)
        assert trav[i] == pytest.approx(tr, rel=1e-12) and rem[i] == pytest.approx(r, abs=1e-9)
        assert dist[i] == pytest.approx(S, rel=1e-14)
    assert not ok[-1] and ok[-2] and seg_ptr[-2] - seg_ptr[-3] > 0


def test_tetra_paths_agree_with_voxel_march(dp):
    """The same box grid traced as voxels and as Kuhn tetrahedra: per box the
    summed path lengths agree to the POINT_EPS nudges (at most 1e-4 m per
    segment boundary of either trace; the last box, cut at the surface
    exit, collects the whole path's difference),
    and the DirectionalPath lists carry the same surface distances."""
    t, _ = _terrains(dp)
    pts, tets, box = _kuhn_mesh(*EDGES)
    vol_t = dp.TetraVolume(pts, tets)
    vol_v = dp.VoxelVolume(*EDGES)
    zen, az = [10.0, 25.0, 40.0, 55.0], [0.0, 70.0, 160.0, 250.0]
    pt = dp.precompute_paths(vol_t, zen, az, t)
    pv = dp.precompute_paths(vol_v, zen, az, t)
    assert len(pt) == len(pv) == 16
    for a, b in zip(pt, pv):
        assert a.valid and b.valid
        assert a.surface_distance == b.surface_distance
        assert a.surface_exit_z == b.surface_exit_z
        per_t, per_v, cnt = {}, {}, {}
        for s in a.segments:
            k = box[s.cell_idx - 1]
            per_t[k] = per_t.get(k, 0.0) + s.distance
            cnt[k] = cnt.get(k, 0) + 1
        for s in b.segments:
            k = s.cell_idx - 1
            per_v[k] = per_v.get(k, 0.0) + s.distance
            cnt[k] = cnt.get(k, 0) + 1
        n_all = len(a.segments) + len(b.segments)
        for k in cnt:
            tol = (n_all + 1) * 1e-4
            assert abs(per_t.get(k, 0.0) - per_v.get(k, 0.0)) <= tol, (k, a.zenith)
        assert abs(a.remaining_rock_distance - b.remaining_rock_distance) <= 2e-2


def test_shallow_mask_and_errors(dp):
    t, _ = _terrains(dp)
    pts, tets, _ = _kuhn_mesh(*EDGES)
    vol = dp.TetraVolume(pts, tets)
    mask = dp.compute_shallow_mask(vol.centroids, t, 60.0)
    s = t.local_surface_height(vol.centroids[:, 0], vol.centroids[:, 1])
    np.testing.assert_array_equal(mask, s - vol.centroids[:, 2] <= 60.0)
    assert 0 < mask.sum() < len(mask)
    assert not dp.compute_shallow_mask(vol.centroids, t, 0.0).any()
    with pytest.raises(ValueError):
        dp.TetraVolume(pts, tets - 1)
    with pytest.raises(ValueError):
        dp.precompute_paths(vol, [10.0], [0.0], dp.flat_surface(100.0))

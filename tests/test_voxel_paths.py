"""Directional paths through a voxel volume (trace_path(::VoxelVolume),
examples/lvd_tomography.jl:583-779): the library's host march against the
oracle's restatement, segment by segment (host logic, no device)."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module", autouse=True)
def library():
    import build  # diffpumas.jl_gb300/build.py: the host march lives in libdpgpu
    build.build()


def test_march_matches_oracle_exactly():
    import dpgpu
    import voxel_paths as ref
    rng = np.random.default_rng(3)
    xe = np.cumsum(np.concatenate([[-300.0], rng.uniform(10.0, 40.0, 17)]))
    ye = np.cumsum(np.concatenate([[-250.0], rng.uniform(15.0, 35.0, 15)]))
    ze = np.cumsum(np.concatenate([[0.0], rng.uniform(10.0, 30.0, 12)]))
    vol = dpgpu.VoxelVolume(xe, ye, ze)
    zen = list(rng.uniform(0.0, 80.0, 40)) + [0.0, 45.0, 89.0]
    az = list(rng.uniform(0.0, 360.0, 3)) + [0.0, 90.0]
    surf = dpgpu.flat_surface(450.0)
    paths = dpgpu.precompute_paths(vol, zen, az, surf)
    k = 0
    for t in zen:
        for p in az:
            path = paths[k]
            k += 1
            assert path.zenith == t and path.azimuth == p
            dist, ok, exit_z = surf(t, p)
            cells, lens, traveled = ref.trace_path((list(xe), list(ye), list(ze)), t, p, dist)
            assert [s.cell_idx - 1 for s in path.segments] == cells
            assert [s.distance for s in path.segments] == lens
            assert path.distance_in_volume == traveled
            assert path.remaining_rock_distance == max(0.0, dist - traveled)
            assert path.surface_distance == dist and path.surface_exit_z == exit_z


def test_invalid_directions():
    import dpgpu
    vol = dpgpu.VoxelVolume([-10.0, 0.0, 10.0], [-10.0, 10.0], [0.0, 5.0, 10.0])
    path = dpgpu.trace_path(vol, 100.0, 0.0, dpgpu.flat_surface(100.0))
    assert not path.valid and path.segments == [] and math.isnan(path.surface_distance)
    path = dpgpu.trace_path(vol, 0.0, 0.0, dpgpu.flat_surface(100.0))
    assert path.valid and len(path.segments) == 2 and path.remaining_rock_distance > 89.0

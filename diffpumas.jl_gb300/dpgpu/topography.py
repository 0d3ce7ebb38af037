"""Terrain and tetrahedral-mesh geometry for directional paths (libdpgpu
host code): the elevation map of src/Turtle.jl:455-640, the surface-exit
search of examples/lvd_tomography.jl:214-252, the ray-triangle test of
src/TriangleIntersect.jl and trace_path(::TetraVolume)
(examples/lvd_tomography.jl:380-528, 694-736).  The tetrahedral mesh is an
input: the reference builds it with TetGen, which is not part of this
library."""
import ctypes as C
import math

import numpy as np

from ._lib import DpElevationMap, DpTerrain, DpTetraMesh, check, load


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


class ElevationMap:
    """Turtle ElevationMap (src/Turtle.jl:455-501): nx x ny nodes spanning
    x_range and y_range; map_create fills every node with z_range[0]."""

    def __init__(self, nx, ny, x_range, y_range, z_range=(0.0, 1.0), data=None):
        if nx <= 0 or ny <= 0:
            raise ValueError("invalid map dimensions")
        if z_range[0] == z_range[1]:
            raise ValueError("zero z range")
        self.nx, self.ny = int(nx), int(ny)
        self.x0, self.y0 = float(x_range[0]), float(y_range[0])
        self.dx = (x_range[1] - x_range[0]) / (nx - 1) if nx > 1 else 0.0
        self.dy = (y_range[1] - y_range[0]) / (ny - 1) if ny > 1 else 0.0
        self.data = np.full((self.ny, self.nx), float(z_range[0])) if data is None \
            else _f64(np.asarray(data).reshape(self.ny, self.nx)).copy()

    def fill(self, ix, iy, elevation):
        """map_fill (src/Turtle.jl:503-507); 0-based node indices."""
        if not (0 <= ix < self.nx and 0 <= iy < self.ny):
            raise ValueError("node indices out of range")
        self.data[iy, ix] = float(elevation)

    def node(self, ix, iy):
        """map_node (src/Turtle.jl:509-517): (x, y, z) of a node."""
        if not (0 <= ix < self.nx and 0 <= iy < self.ny):
            raise ValueError("node indices out of range")
        return self.x0 + ix * self.dx, self.y0 + iy * self.dy, float(self.data[iy, ix])

    def _c(self):
        self._z = np.ascontiguousarray(self.data, np.float64)
        return DpElevationMap(self.nx, self.ny, self.x0, self.y0, self.dx, self.dy,
                              self._z.ctypes.data)

    def elevation(self, x, y):
        """map_elevation (src/Turtle.jl:520-557): (z, inside), vectorised."""
        x, y = np.broadcast_arrays(_f64(np.atleast_1d(x)), _f64(np.atleast_1d(y)))
        x, y = _f64(x), _f64(y)
        z, inside = np.zeros(len(x)), np.zeros(len(x), np.int32)
        m = self._c()
        check(load().dp_map_elevation(C.byref(m), len(x), x.ctypes.data, y.ctypes.data,
                                      z.ctypes.data, inside.ctypes.data))
        return z, inside.astype(bool)

    def gradient(self, x, y):
        """map_gradient (src/Turtle.jl:559-634): (gx, gy, inside), vectorised."""
        x, y = np.broadcast_arrays(_f64(np.atleast_1d(x)), _f64(np.atleast_1d(y)))
        x, y = _f64(x), _f64(y)
        gx, gy, inside = np.zeros(len(x)), np.zeros(len(x)), np.zeros(len(x), np.int32)
        m = self._c()
        check(load().dp_map_gradient(C.byref(m), len(x), x.ctypes.data, y.ctypes.data,
                                     gx.ctypes.data, gy.ctypes.data, inside.ctypes.data))
        return gx, gy, inside.astype(bool)


class Terrain:
    """The terrain above a detector at the origin: an elevation map in
    `xy_scale` map units per metre (the LVD map is in km) and the detector
    elevation (examples/lvd_tomography.jl:214-217), with the surface-exit
    search's step and range (:148, :219-252).  Calling it with (zenith,
    azimuth) gives (slant distance, valid, exit altitude), the role of
    ray_surface_exit_distance in precompute_paths."""

    def __init__(self, emap, detector_elevation=963.0, xy_scale=1e-3, step=40.0,
                 max_distance=25000.0):
        self.map, self.detector_elevation = emap, float(detector_elevation)
        self.xy_scale, self.step, self.max_distance = float(xy_scale), float(step), \
            float(max_distance)

    def _c(self):
        return DpTerrain(self.map._c(), self.xy_scale, self.detector_elevation, self.step,
                         self.max_distance)

    def local_surface_height(self, x, y):
        """Surface height above the detector at local metres; NaN off the map."""
        z, inside = self.map.elevation(np.asarray(x, np.float64) * self.xy_scale,
                                       np.asarray(y, np.float64) * self.xy_scale)
        return np.where(inside, z - self.detector_elevation, np.nan)

    def surface_exit(self, zeniths, azimuths):
        """(distance, exit_z, ok) per direction (dp_surface_exit)."""
        zen, az = _f64(np.atleast_1d(zeniths)), _f64(np.atleast_1d(azimuths))
        n = len(zen)
        d, z, ok = np.zeros(n), np.zeros(n), np.zeros(n, np.int32)
        t = self._c()
        check(load().dp_surface_exit(C.byref(t), n, zen.ctypes.data, az.ctypes.data,
                                     d.ctypes.data, z.ctypes.data, ok.ctypes.data))
        return d, z, ok.astype(bool)

    def __call__(self, zenith, azimuth):
        d, z, ok = self.surface_exit([zenith], [azimuth])
        return (float(d[0]), True, float(z[0])) if ok[0] else (math.nan, False, math.nan)


def ray_triangle_intersect(origin, direction, p1, p2, p3):
    """intersect (src/TriangleIntersect.jl:78-115): (hit, distance, point)."""
    a = [_f64(v) for v in (origin, direction, p1, p2, p3)]
    t = C.c_double()
    ip = np.zeros(3)
    hit = load().dp_ray_triangle(*[v.ctypes.data for v in a], C.byref(t), ip.ctypes.data)
    return bool(hit), t.value, ip


class TetraVolume:
    """A tetrahedral sensitivity volume (examples/lvd_tomography.jl:172-179):
    points (n x 3, metres, the detector at the origin), tets (m x 4, 1-based
    point indices as TetGen writes them), the face-neighbour table
    (build_tetra_neighbors), centroids (tetra_centroids) and the shallow
    mask."""

    def __init__(self, points, tets, shallow_mask=None):
        self.points = _f64(np.asarray(points, np.float64).reshape(-1, 3))
        self.tets = np.ascontiguousarray(np.asarray(tets).reshape(-1, 4), np.int32)
        if self.tets.size and (self.tets.min() < 1 or self.tets.max() > len(self.points)):
            raise ValueError("Expected one-based TetGen connectivity within pointlist")
        self.neighbors = np.zeros((len(self.tets), 4), np.int32)
        m = self._c()
        check(load().dp_tetra_neighbors(C.byref(m), self.neighbors.ctypes.data))
        self.centroids = self.points[self.tets - 1].sum(axis=1) / 4.0
        self.shallow_mask = np.zeros(len(self.tets), bool) if shallow_mask is None \
            else np.asarray(shallow_mask, bool)

    @property
    def n_cells(self):
        return len(self.tets)

    def _c(self):
        return DpTetraMesh(len(self.points), self.points.ctypes.data, len(self.tets),
                           self.tets.ctypes.data)


def compute_shallow_mask(centroids, terrain, porous_top_thickness):
    """compute_shallow_mask (examples/lvd_tomography.jl:395-408): cells whose
    centroid lies within porous_top_thickness below the terrain."""
    c = np.asarray(centroids, np.float64).reshape(-1, 3)
    if porous_top_thickness <= 0.0:
        return np.zeros(len(c), bool)
    s = terrain.local_surface_height(c[:, 0], c[:, 1])
    with np.errstate(invalid="ignore"):
        return np.isfinite(s) & (s - c[:, 2] <= porous_top_thickness)


def trace_tetra_paths(volume, terrain, zeniths, azimuths):
    """trace_path(::TetraVolume) of every direction (dp_tetra_trace):
    (seg_ptr, cells (1-based), lengths, traveled, surface distance,
    remaining rock, exit z, valid)."""
    zen, az = _f64(np.atleast_1d(zeniths)), _f64(np.atleast_1d(azimuths))
    n = len(zen)
    seg_ptr = np.zeros(n + 1, np.int64)
    out = [np.zeros(max(n, 1)) for _ in range(4)]
    valid = np.zeros(max(n, 1), np.int32)
    m, t = volume._c(), terrain._c()
    lib = load()
    args = (None, C.byref(m), volume.neighbors.ctypes.data, C.byref(t), n, zen.ctypes.data,
            az.ctypes.data, seg_ptr.ctypes.data)
    check(lib.dp_tetra_trace(*args, None, None, 0, None, None, None, None, None))
    k = int(seg_ptr[-1])
    cells, lens = np.zeros(max(k, 1), np.int32), np.zeros(max(k, 1))
    check(lib.dp_tetra_trace(*args, cells.ctypes.data, lens.ctypes.data, k,
                             *[o.ctypes.data for o in out], valid.ctypes.data))
    return (seg_ptr, cells[:k], lens[:k], out[0][:n], out[1][:n], out[2][:n], out[3][:n],
            valid[:n].astype(bool))

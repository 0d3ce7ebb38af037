"""Pure-Python restatement of the voxel march of examples/lvd_tomography.jl
(voxel_cell_indices :583-594, distance_to_voxel_boundary :596-627,
trace_path(::VoxelVolume) :738-779).  TEST INFRASTRUCTURE ONLY: the checker
of the library's dp_voxel_trace."""
import bisect
import math

POINT_EPS = 1e-4  # examples/lvd_tomography.jl:147


def _cell(edges, x, y, z):
    xe, ye, ze = edges
    if x < xe[0] or x > xe[-1] or y < ye[0] or y > ye[-1] or z < ze[0] or z > ze[-1]:
        return None
    idx = []
    for e, v in ((xe, x), (ye, y), (ze, z)):
        i = bisect.bisect_right(e, v) - 1           # searchsortedlast, 0-based
        idx.append(min(max(i, 0), len(e) - 2))
    return tuple(idx)


def _boundary(edges, x, y, z, d):
    c = _cell(edges, x, y, z)
    if c is None:
        return 0.0
    t_min = math.inf
    for e, p, u, i in zip(edges, (x, y, z), d, c):
        if abs(u) > 1e-10:
            t = (e[i + 1] - p) / u if u > 0 else (e[i] - p) / u
            if t > 1e-10:
                t_min = min(t_min, t)
    return t_min if math.isfinite(t_min) else 0.0


def trace_path(edges, zenith, azimuth, surface):
    """(cells 0-based, lengths, traveled) of the march to slant distance surface."""
    th, ph = zenith * (math.pi / 180.0), azimuth * (math.pi / 180.0)
    dh = math.sin(th)
    d = (dh * math.sin(ph), dh * math.cos(ph), math.cos(th))
    nx, ny = len(edges[0]) - 1, len(edges[1]) - 1
    x, y, z = d[0] * POINT_EPS, d[1] * POINT_EPS, d[2] * POINT_EPS
    traveled = POINT_EPS
    cells, lens = [], []
    while traveled < surface - POINT_EPS:
        c = _cell(edges, x, y, z)
        if c is None:
            break
        dist = _boundary(edges, x, y, z, d)
        if not math.isfinite(dist) or dist <= 0.0:
            break
        remaining = surface - traveled
        step = min(dist, remaining)
        if step > 1e-8:
            cells.append(c[0] + nx * (c[1] + ny * c[2]))
            lens.append(step)
            traveled += step
        if dist >= remaining - 1e-6:
            break
        x += d[0] * (step + POINT_EPS)
        y += d[1] * (step + POINT_EPS)
        z += d[2] * (step + POINT_EPS)
    return cells, lens, traveled

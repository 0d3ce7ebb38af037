"""TEST INFRASTRUCTURE ONLY -- the oracle's pure-Python restatement of the
terrain and tetrahedral-mesh geometry of the directional paths:
map_elevation (src/Turtle.jl:520-557), local_surface_height and
ray_surface_exit_distance (examples/lvd_tomography.jl:214-252), intersect
(src/TriangleIntersect.jl:78-115) and the tetrahedral walk of
examples/lvd_tomography.jl:410-528, 694-736.  Small cases only."""
import math

import numpy as np

POINT_EPS = 1e-4  # examples/lvd_tomography.jl:147


def map_elevation(nx, ny, x0, y0, dx, dy, data, x, y):
    """src/Turtle.jl:520-557; data[iy][ix]."""
    if math.isnan(x) or math.isnan(y):
        return 0.0, False
    hx, hy = (x - x0) / dx, (y - y0) / dy
    if hx > nx - 1 or hx < 0 or hy > ny - 1 or hy < 0:
        return 0.0, False
    ix, iy = math.floor(hx), math.floor(hy)
    if ix == nx - 1:
        ix -= 1
        hx = 1.0
    else:
        hx -= ix
    if iy == ny - 1:
        iy -= 1
        hy = 1.0
    else:
        hy -= iy
    z00, z10 = data[iy][ix], data[iy][ix + 1]
    z01, z11 = data[iy + 1][ix], data[iy + 1][ix + 1]
    return (z00 * (1.0 - hx) * (1.0 - hy) + z01 * (1.0 - hx) * hy + z10 * hx * (1.0 - hy) +
            z11 * hx * hy), True


class Terrain:
    def __init__(self, nx, ny, x0, y0, dx, dy, data, detector_elevation, xy_scale=1e-3,
                 step=40.0, max_distance=25000.0):
        self.m = (nx, ny, x0, y0, dx, dy, [list(map(float, r)) for r in data])
        self.det, self.scale, self.step, self.max = detector_elevation, xy_scale, step, \
            max_distance

    def height(self, x, y):
        """local_surface_height (examples/lvd_tomography.jl:214-217)."""
        z, inside = map_elevation(*self.m, x * self.scale, y * self.scale)
        return z - self.det if inside else math.nan

    def exit(self, d):
        """ray_surface_exit_distance (examples/lvd_tomography.jl:219-252)."""
        if d[2] <= 0.0:
            return math.nan, False, math.nan
        prev = 0.0
        for k in range(1, int(math.floor(self.max / self.step + 1e-9)) + 1):
            s = k * self.step
            zs = self.height(d[0] * s, d[1] * s)
            if not math.isfinite(zs):
                return math.nan, False, math.nan
            if d[2] * s > zs:
                lo, hi = prev, s
                for _ in range(40):
                    mid = 0.5 * (lo + hi)
                    if d[2] * mid > self.height(d[0] * mid, d[1] * mid):
                        hi = mid
                    else:
                        lo = mid
                se = 0.5 * (lo + hi)
                return se, True, d[2] * se
            prev = s
        return math.nan, False, math.nan


def direction_vector(zenith, azimuth):
    """src/Tomography.jl:229-234."""
    th, ph = math.radians(zenith), math.radians(azimuth)
    dh = math.sin(th)
    return (dh * math.sin(ph), dh * math.cos(ph), math.cos(th))


def _sub(a, b):
    return [a[0] - b[0], a[1] - b[1], a[2] - b[2]]


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def intersect(o, d, v0, v1, v2):
    """src/TriangleIntersect.jl:78-115: (hit, t, point)."""
    eps = 1e-10
    e1, e2 = _sub(v1, v0), _sub(v2, v0)
    h = _cross(d, e2)
    a = _dot(e1, h)
    if abs(a) < eps:
        return False, math.inf, None
    f = 1.0 / a
    s = _sub(o, v0)
    u = f * _dot(s, h)
    if u < 0.0 or u > 1.0:
        return False, math.inf, None
    q = _cross(s, e1)
    v = f * _dot(d, q)
    if v < 0.0 or u + v > 1.0:
        return False, math.inf, None
    t = f * _dot(e2, q)
    if t > eps:
        return True, t, [o[0] + t * d[0], o[1] + t * d[1], o[2] + t * d[2]]
    return False, math.inf, None


def tolerant_hit(o, d, a, b, c):
    """examples/lvd_tomography.jl:485-503."""
    e1, e2 = _sub(b, a), _sub(c, a)
    n = _cross(e1, e2)
    den = _dot(n, d)
    if not abs(den) > 1e-12 * math.sqrt(_dot(n, n)):
        return None
    dist = _dot(n, _sub(a, o)) / den
    if not dist > 1e-8:
        return None
    off = [o[k] + dist * d[k] - a[k] for k in range(3)]
    aa, ab, bb = _dot(e1, e1), _dot(e1, e2), _dot(e2, e2)
    det = aa * bb - ab * ab
    if not det > 0:
        return None
    u = (bb * _dot(off, e1) - ab * _dot(off, e2)) / det
    v = (aa * _dot(off, e2) - ab * _dot(off, e1)) / det
    if not min(u, v, 1 - u - v) >= -1e-10:
        return None
    return dist, [o[k] + dist * d[k] for k in range(3)]


FACES = ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3))  # tetra_face_indices, :415-422


def tetra_neighbors(tets):
    """build_tetra_neighbors (examples/lvd_tomography.jl:431-453); 1-based."""
    faces = {}
    for t, tv in enumerate(tets):
        for f, fc in enumerate(FACES):
            key = tuple(sorted(int(tv[i]) for i in fc))
            faces.setdefault(key, []).append((t, f))
    nb = np.zeros((len(tets), 4), np.int32)
    for entries in faces.values():
        if len(entries) == 2:
            (t1, f1), (t2, f2) = entries
            nb[t1, f1] = t2 + 1
            nb[t2, f2] = t1 + 1
    return nb


def point_in_tet(p, tv, pts, atol=1e-8):
    """point_in_tetrahedron (examples/lvd_tomography.jl:455-470)."""
    a = pts[tv[0] - 1]
    mat = np.column_stack([pts[tv[1] - 1] - a, pts[tv[2] - 1] - a, pts[tv[3] - 1] - a])
    if abs(np.linalg.det(mat)) < atol:
        return False
    b = np.linalg.solve(mat, np.asarray(p) - a)
    return b[0] >= -atol and b[1] >= -atol and b[2] >= -atol and b.sum() <= 1.0 + atol


def trace_tetra(pts, tets, nb, terrain, zenith, azimuth):
    """trace_path(::TetraVolume) (examples/lvd_tomography.jl:694-736):
    (segments [(cell, length)], traveled, surface distance, remaining, exit z, valid)."""
    d = direction_vector(zenith, azimuth)
    S, ok, ez = terrain.exit(d)
    if not ok:
        return [], math.nan, math.nan, math.nan, math.nan, False
    p = [d[0] * POINT_EPS, d[1] * POINT_EPS, d[2] * POINT_EPS]
    cur = next((t + 1 for t in range(len(tets)) if point_in_tet(p, tets[t], pts)), 0)
    segs = []
    trav = POINT_EPS if cur else 0.0
    while cur and trav < S - POINT_EPS:
        tv = tets[cur - 1]
        best, bf, bp = math.inf, 0, p
        for f, fc in enumerate(FACES):
            a, b, c = (list(pts[tv[i] - 1]) for i in fc)
            hit, t, ip = intersect(p, d, a, b, c)
            cand = (t, ip) if hit else tolerant_hit(p, d, a, b, c)
            if cand is not None and cand[0] > 1e-8 and cand[0] < best:
                best, bf, bp = cand[0], f + 1, cand[1]
        if bf == 0 or not math.isfinite(best):
            break
        remaining = S - trav
        step = min(best, remaining)
        if step > 1e-8:
            segs.append((cur, step))
            trav += step
        if best >= remaining - 1e-6:
            break
        nxt = int(nb[cur - 1, bf - 1])
        if nxt == 0:
            break
        p = [bp[k] + d[k] * POINT_EPS for k in range(3)]
        cur = nxt
    return segs, trav, S, max(0.0, S - trav), ez, True

// topo_trace.cu -- terrain and tetrahedral-mesh geometry for directional
// paths: the elevation map of src/Turtle.jl:455-640 (map_elevation,
// map_gradient), the surface-exit search of examples/lvd_tomography.jl:214-252
// (local_surface_height, ray_surface_exit_distance), the ray-triangle test of
// src/TriangleIntersect.jl:78-115 and the tetrahedral walk of
// examples/lvd_tomography.jl:410-528, 694-736 (tetra_face_indices,
// build_tetra_neighbors, point_in_tetrahedron,
// find_tetrahedron_containing_point, tolerant_tetra_face_hit,
// nearest_tetra_face_intersection, trace_path(::TetraVolume)).  Host code:
// it runs once per geometry and produces the segment lists (cell, length)
// the water-fraction CSDA model and the fixed-path MC consume.  FP64 with the
// reference's operations.  The mesh is an input (the reference builds it
// with TetGen, which this library does not include).
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <vector>

#include "internal.h"

namespace {

constexpr double kPointEps = 1e-4;  // POINT_EPS (examples/lvd_tomography.jl:147)

// map_elevation (src/Turtle.jl:520-557); false outside the map.
bool map_elev(const dp_elevation_map& m, double x, double y, double* z) {
  if (std::isnan(x) || std::isnan(y)) return false;
  double hx = (x - m.x0) / m.dx, hy = (y - m.y0) / m.dy;
  if (hx > m.nx - 1 || hx < 0 || hy > m.ny - 1 || hy < 0) return false;
  int ix = int(std::floor(hx)), iy = int(std::floor(hy));
  if (ix == m.nx - 1) {
    ix -= 1;
    hx = 1.0;
  } else {
    hx -= ix;
  }
  if (iy == m.ny - 1) {
    iy -= 1;
    hy = 1.0;
  } else {
    hy -= iy;
  }
  auto Z = [&](int i, int j) { return m.z[size_t(j) * m.nx + i]; };
  const double z00 = Z(ix, iy), z10 = Z(ix + 1, iy), z01 = Z(ix, iy + 1), z11 = Z(ix + 1, iy + 1);
  *z = z00 * (1.0 - hx) * (1.0 - hy) + z01 * (1.0 - hx) * hy + z10 * hx * (1.0 - hy) +
       z11 * hx * hy;
  return true;
}

// map_gradient (src/Turtle.jl:559-634): adaptive two-cell stencil.
bool map_grad(const dp_elevation_map& m, double x, double y, double* gx, double* gy) {
  if (std::isnan(x) || std::isnan(y)) return false;
  double hx = (x - m.x0) / m.dx, hy = (y - m.y0) / m.dy;
  if (hx > m.nx - 1 || hx < 0 || hy > m.ny - 1 || hy < 0) return false;
  int ix = int(std::floor(hx)), iy = int(std::floor(hy));
  if (ix == m.nx - 1) {
    ix -= 1;
    hx = 1.0;
  } else {
    hx -= ix;
  }
  if (iy == m.ny - 1) {
    iy -= 1;
    hy = 1.0;
  } else {
    hy -= iy;
  }
  auto Z = [&](int i, int j) { return m.z[size_t(j) * m.nx + i]; };
  const double z00 = Z(ix, iy), z10 = Z(ix + 1, iy), z01 = Z(ix, iy + 1), z11 = Z(ix + 1, iy + 1);
  if (hx <= 0.5) {
    const double g1 = (z10 - z00) * (1.0 - hy) + (z11 - z01) * hy;
    if (ix == 0) {
      *gx = g1 / m.dx;
    } else {
      const double g0 = (z00 - Z(ix - 1, iy)) * (1.0 - hy) + (z01 - Z(ix - 1, iy + 1)) * hy;
      const double a = hx + 0.5;
      *gx = (g0 * (1.0 - a) + g1 * a) / m.dx;
    }
  } else {
    const double g0 = (z10 - z00) * (1.0 - hy) + (z11 - z01) * hy;
    if (ix == m.nx - 2) {
      *gx = g0 / m.dx;
    } else {
      const double g1 = (Z(ix + 2, iy) - z10) * (1.0 - hy) + (Z(ix + 2, iy + 1) - z11) * hy;
      const double a = hx - 0.5;
      *gx = (g0 * (1.0 - a) + g1 * a) / m.dx;
    }
  }
  if (hy <= 0.5) {
    const double g1 = (z01 - z00) * (1.0 - hx) + (z11 - z10) * hx;
    if (iy == 0) {
      *gy = g1 / m.dy;
    } else {
      const double g0 = (z00 - Z(ix, iy - 1)) * (1.0 - hx) + (z10 - Z(ix + 1, iy - 1)) * hx;
      const double a = hy + 0.5;
      *gy = (g0 * (1.0 - a) + g1 * a) / m.dy;
    }
  } else {
    const double g0 = (z01 - z00) * (1.0 - hx) + (z11 - z10) * hx;
    if (iy == m.ny - 2) {
      *gy = g0 / m.dy;
    } else {
      const double g1 = (Z(ix, iy + 2) - z01) * (1.0 - hx) + (Z(ix + 1, iy + 2) - z11) * hx;
      const double a = hy - 0.5;
      *gy = (g0 * (1.0 - a) + g1 * a) / m.dy;
    }
  }
  return true;
}

// local_surface_height (examples/lvd_tomography.jl:214-217): the terrain
// above the detector at local metres (x, y), NaN outside the map.
double surface_height(const dp_terrain& t, double x, double y) {
  double z;
  if (!map_elev(t.map, x * t.xy_scale, y * t.xy_scale, &z)) return NAN;
  return z - t.detector_elevation;
}

// ray_surface_exit_distance (examples/lvd_tomography.jl:219-252): march in
// steps of t.step up to t.max_distance, then 40 bisections.
bool surface_exit(const dp_terrain& t, const double d[3], double* s_exit, double* z_exit) {
  if (d[2] <= 0.0) return false;
  double prev = 0.0;
  // the reference's range step:step:max (an exact count of steps)
  const long n = long(std::floor(t.max_distance / t.step + 1e-9));
  for (long k = 1; k <= n; ++k) {
    const double s = double(k) * t.step;
    const double zs = surface_height(t, d[0] * s, d[1] * s);
    if (!std::isfinite(zs)) return false;
    if (d[2] * s > zs) {
      double lo = prev, hi = s;
      for (int it = 0; it < 40; ++it) {
        const double mid = 0.5 * (lo + hi);
        const double ms = surface_height(t, d[0] * mid, d[1] * mid);
        if (d[2] * mid > ms) hi = mid;
        else lo = mid;
      }
      *s_exit = 0.5 * (lo + hi);
      *z_exit = d[2] * *s_exit;
      return true;
    }
    prev = s;
  }
  return false;
}

using V3 = std::array<double, 3>;
V3 sub3(const V3& a, const V3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
V3 cross3(const V3& a, const V3& b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
double dot3(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// intersect (src/TriangleIntersect.jl:78-115), Moller-Trumbore.
bool ray_triangle(const V3& o, const V3& d, const V3& v0, const V3& v1, const V3& v2, double* t,
                  V3* ip) {
  const double eps = 1e-10;
  const V3 e1 = sub3(v1, v0), e2 = sub3(v2, v0);
  const V3 h = cross3(d, e2);
  const double a = dot3(e1, h);
  if (std::fabs(a) < eps) return false;
  const double f = 1.0 / a;
  const V3 s = sub3(o, v0);
  const double u = f * dot3(s, h);
  if (u < 0.0 || u > 1.0) return false;
  const V3 q = cross3(s, e1);
  const double v = f * dot3(d, q);
  if (v < 0.0 || u + v > 1.0) return false;
  const double tt = f * dot3(e2, q);
  if (!(tt > eps)) return false;
  *t = tt;
  *ip = {o[0] + tt * d[0], o[1] + tt * d[1], o[2] + tt * d[2]};
  return true;
}

// tolerant_tetra_face_hit (examples/lvd_tomography.jl:485-503): the plane
// hit with barycentric coordinates down to -1e-10 (shared-edge hits).
bool tolerant_hit(const V3& o, const V3& d, const V3& a, const V3& b, const V3& c, double* t,
                  V3* ip) {
  const V3 e1 = sub3(b, a), e2 = sub3(c, a);
  const V3 n = cross3(e1, e2);
  const double den = dot3(n, d);
  if (!(std::fabs(den) > 1e-12 * std::sqrt(dot3(n, n)))) return false;
  const double dist = dot3(n, sub3(a, o)) / den;
  if (!(dist > 1e-8)) return false;
  const V3 off = {o[0] + dist * d[0] - a[0], o[1] + dist * d[1] - a[1], o[2] + dist * d[2] - a[2]};
  const double aa = dot3(e1, e1), ab = dot3(e1, e2), bb = dot3(e2, e2);
  const double det = aa * bb - ab * ab;
  if (!(det > 0)) return false;
  const double u = (bb * dot3(off, e1) - ab * dot3(off, e2)) / det;
  const double v = (aa * dot3(off, e2) - ab * dot3(off, e1)) / det;
  if (!(std::min(std::min(u, v), 1 - u - v) >= -1e-10)) return false;
  *t = dist;
  *ip = {o[0] + dist * d[0], o[1] + dist * d[1], o[2] + dist * d[2]};
  return true;
}

// tetra_face_indices (examples/lvd_tomography.jl:415-422): local vertex
// triples of faces 1..4.
constexpr int kFace[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

V3 point(const dp_tetra_mesh& m, int one_based) {
  const double* p = m.points + 3 * size_t(one_based - 1);
  return {p[0], p[1], p[2]};
}

// point_in_tetrahedron (examples/lvd_tomography.jl:455-470): barycentric
// coordinates from the 3x3 system (LU with partial pivoting), atol 1e-8.
bool point_in_tet(const dp_tetra_mesh& m, const int32_t* tet, const V3& p) {
  const double atol = 1e-8;
  const V3 a = point(m, tet[0]);
  double A[3][3], r[3];
  for (int c = 0; c < 3; ++c) {
    const V3 v = point(m, tet[c + 1]);
    for (int k = 0; k < 3; ++k) A[k][c] = v[k] - a[k];
  }
  for (int k = 0; k < 3; ++k) r[k] = p[k] - a[k];
  // determinant and solve by Gaussian elimination with partial pivoting
  double det = 1.0;
  int perm[3] = {0, 1, 2};
  for (int j = 0; j < 3; ++j) {
    int piv = j;
    for (int i = j + 1; i < 3; ++i)
      if (std::fabs(A[i][j]) > std::fabs(A[piv][j])) piv = i;
    if (piv != j) {
      for (int k = 0; k < 3; ++k) std::swap(A[j][k], A[piv][k]);
      std::swap(r[j], r[piv]);
      std::swap(perm[j], perm[piv]);
      det = -det;
    }
    det *= A[j][j];
    if (A[j][j] == 0.0) return false;
    const double inv = 1.0 / A[j][j];
    for (int i = j + 1; i < 3; ++i) {
      const double l = A[i][j] * inv;
      for (int k = j; k < 3; ++k) A[i][k] -= l * A[j][k];
      r[i] -= l * r[j];
    }
  }
  if (std::fabs(det) < atol) return false;
  // back substitution in LAPACK's column order (dtrsv, upper, no transpose)
  double b[3] = {r[0], r[1], r[2]};
  for (int j = 2; j >= 0; --j) {
    b[j] = b[j] / A[j][j];
    for (int i = j - 1; i >= 0; --i) b[i] -= b[j] * A[i][j];
  }
  return b[0] >= -atol && b[1] >= -atol && b[2] >= -atol && b[0] + b[1] + b[2] <= 1.0 + atol;
}

// find_tetrahedron_containing_point (examples/lvd_tomography.jl:472-481):
// the first tetrahedron (1-based) containing p, 0 if none, scanning the
// candidates in index order (every path starts POINT_EPS from the origin,
// so only tetrahedra whose bounding box reaches that ball can hold it).
long find_tet(const dp_tetra_mesh& m, const std::vector<long>& cand, const V3& p) {
  for (long t : cand)
    if (point_in_tet(m, m.tets + 4 * t, p)) return t + 1;
  return 0;
}
std::vector<long> start_candidates(const dp_tetra_mesh& m) {
  const double r = 2.0 * kPointEps + 1e-6;
  std::vector<long> out;
  for (long t = 0; t < m.n_tets; ++t) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int v = 0; v < 4; ++v) {
      const V3 q = point(m, m.tets[4 * t + v]);
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], q[k]);
        hi[k] = std::max(hi[k], q[k]);
      }
    }
    if (lo[0] <= r && hi[0] >= -r && lo[1] <= r && hi[1] >= -r && lo[2] <= r && hi[2] >= -r)
      out.push_back(t);
  }
  return out;
}

// nearest_tetra_face_intersection (examples/lvd_tomography.jl:505-527).
int nearest_face(const dp_tetra_mesh& m, long tet, const V3& p, const V3& d, double* best,
                 V3* bp) {
  const int32_t* tv = m.tets + 4 * (tet - 1);
  int face = 0;
  *best = INFINITY;
  *bp = p;
  for (int f = 0; f < 4; ++f) {
    const V3 a = point(m, tv[kFace[f][0]]), b = point(m, tv[kFace[f][1]]),
             c = point(m, tv[kFace[f][2]]);
    double t;
    V3 ip;
    const bool hit = ray_triangle(p, d, a, b, c, &t, &ip) || tolerant_hit(p, d, a, b, c, &t, &ip);
    if (hit && t > 1e-8 && t < *best) {
      face = f + 1;
      *best = t;
      *bp = ip;
    }
  }
  return face;
}

bool check_map(const dp_elevation_map* m) {
  return m && m->z && m->nx >= 2 && m->ny >= 2 && m->dx > 0.0 && m->dy > 0.0;
}
bool check_terrain(const dp_terrain* t) {
  return t && check_map(&t->map) && t->xy_scale > 0.0 && t->step > 0.0 &&
         t->max_distance >= t->step;
}
bool check_mesh(const dp_tetra_mesh* m) {
  if (!m || !m->points || !m->tets || m->n_points < 4 || m->n_tets < 1) return false;
  for (long i = 0; i < 4 * m->n_tets; ++i)
    if (m->tets[i] < 1 || m->tets[i] > m->n_points) return false;
  return true;
}

V3 direction(double zenith, double azimuth) {  // direction_vector, src/Tomography.jl:229-234
  const double th = zenith * (M_PI / 180.0), ph = azimuth * (M_PI / 180.0), dh = std::sin(th);
  return {dh * std::sin(ph), dh * std::cos(ph), std::cos(th)};
}

}  // namespace

using dp::fail;

extern "C" {

int dp_map_elevation(const dp_elevation_map* m, long n, const double* x, const double* y,
                     double* z, int32_t* inside) {
  if (!check_map(m) || n < 0 || (n > 0 && (!x || !y || !z || !inside))) return DP_ERR_ARG;
  for (long i = 0; i < n; ++i) {
    double v = 0.0;
    inside[i] = map_elev(*m, x[i], y[i], &v) ? 1 : 0;
    z[i] = inside[i] ? v : 0.0;
  }
  return DP_OK;
}

int dp_map_gradient(const dp_elevation_map* m, long n, const double* x, const double* y,
                    double* gx, double* gy, int32_t* inside) {
  if (!check_map(m) || n < 0 || (n > 0 && (!x || !y || !gx || !gy || !inside))) return DP_ERR_ARG;
  for (long i = 0; i < n; ++i) {
    double a = 0.0, b = 0.0;
    inside[i] = map_grad(*m, x[i], y[i], &a, &b) ? 1 : 0;
    gx[i] = a;
    gy[i] = b;
  }
  return DP_OK;
}

int dp_ray_triangle(const double* origin, const double* dir, const double* p1, const double* p2,
                    const double* p3, double* distance, double* point) {
  if (!origin || !dir || !p1 || !p2 || !p3 || !distance) return DP_ERR_ARG;
  double t;
  V3 ip;
  const bool hit = ray_triangle({origin[0], origin[1], origin[2]}, {dir[0], dir[1], dir[2]},
                                {p1[0], p1[1], p1[2]}, {p2[0], p2[1], p2[2]},
                                {p3[0], p3[1], p3[2]}, &t, &ip);
  *distance = hit ? t : INFINITY;
  if (point) for (int k = 0; k < 3; ++k) point[k] = hit ? ip[k] : 0.0;
  return hit ? 1 : 0;
}

int dp_surface_exit(const dp_terrain* t, long n_dirs, const double* zenith, const double* azimuth,
                    double* distance, double* exit_z, int32_t* ok) {
  if (!check_terrain(t) || n_dirs < 0 ||
      (n_dirs > 0 && (!zenith || !azimuth || !distance || !exit_z || !ok)))
    return DP_ERR_ARG;
  for (long i = 0; i < n_dirs; ++i) {
    const V3 d = direction(zenith[i], azimuth[i]);
    double s = NAN, z = NAN;
    ok[i] = surface_exit(*t, d.data(), &s, &z) ? 1 : 0;
    distance[i] = ok[i] ? s : NAN;
    exit_z[i] = ok[i] ? z : NAN;
  }
  return DP_OK;
}

int dp_tetra_neighbors(const dp_tetra_mesh* m, int32_t* neighbors) {
  if (!check_mesh(m) || !neighbors) return DP_ERR_ARG;
  std::map<std::array<int32_t, 3>, std::vector<std::pair<long, int>>> faces;
  for (long t = 0; t < m->n_tets; ++t) {
    const int32_t* tv = m->tets + 4 * t;
    for (int f = 0; f < 4; ++f) {
      std::array<int32_t, 3> key = {tv[kFace[f][0]], tv[kFace[f][1]], tv[kFace[f][2]]};
      std::sort(key.begin(), key.end());
      faces[key].push_back({t, f});
    }
  }
  std::fill(neighbors, neighbors + 4 * m->n_tets, 0);
  for (const auto& kv : faces)
    if (kv.second.size() == 2) {
      const auto& a = kv.second[0];
      const auto& b = kv.second[1];
      neighbors[4 * a.first + a.second] = int32_t(b.first + 1);
      neighbors[4 * b.first + b.second] = int32_t(a.first + 1);
    }
  return DP_OK;
}

int dp_tetra_trace(dp_ctx* ctx, const dp_tetra_mesh* m, const int32_t* neighbors,
                   const dp_terrain* terrain, long n_dirs, const double* zenith,
                   const double* azimuth, int64_t* seg_ptr, int32_t* seg_cell,
                   double* seg_length, int64_t seg_cap, double* traveled_out,
                   double* surface_distance, double* remaining_rock, double* exit_z,
                   int32_t* valid) {
  if (!check_mesh(m) || !neighbors || !check_terrain(terrain))
    return fail(ctx, DP_ERR_ARG, "bad mesh, neighbour table or terrain");
  if (n_dirs < 0 || (n_dirs > 0 && (!zenith || !azimuth || !seg_ptr)))
    return fail(ctx, DP_ERR_ARG, "bad direction arrays");
  std::vector<int32_t> cells;
  std::vector<double> lens;
  const std::vector<long> cand = start_candidates(*m);
  seg_ptr[0] = 0;
  for (long i = 0; i < n_dirs; ++i) {
    const V3 d = direction(zenith[i], azimuth[i]);
    double S = NAN, ez = NAN, trav = NAN, rem = NAN;
    const bool ok = surface_exit(*terrain, d.data(), &S, &ez);
    if (ok) {
      V3 p = {d[0] * kPointEps, d[1] * kPointEps, d[2] * kPointEps};
      long tet = find_tet(*m, cand, p);
      trav = tet ? kPointEps : 0.0;
      for (long guard = 0; tet && trav < S - kPointEps && guard < 100000000; ++guard) {
        double dist;
        V3 ip;
        const int face = nearest_face(*m, tet, p, d, &dist, &ip);
        if (face == 0 || !std::isfinite(dist)) break;
        const double remaining = S - trav;
        const double step = std::min(dist, remaining);
        if (step > 1e-8) {
          cells.push_back(int32_t(tet));
          lens.push_back(step);
          trav += step;
        }
        if (dist >= remaining - 1e-6) break;
        const int32_t next = neighbors[4 * (tet - 1) + face - 1];
        if (next == 0) break;
        p = {ip[0] + d[0] * kPointEps, ip[1] + d[1] * kPointEps, ip[2] + d[2] * kPointEps};
        tet = next;
      }
      rem = std::max(0.0, S - trav);
    }
    seg_ptr[i + 1] = int64_t(cells.size());
    if (traveled_out) traveled_out[i] = ok ? trav : NAN;
    if (surface_distance) surface_distance[i] = ok ? S : NAN;
    if (remaining_rock) remaining_rock[i] = ok ? rem : NAN;
    if (exit_z) exit_z[i] = ok ? ez : NAN;
    if (valid) valid[i] = ok ? 1 : 0;
  }
  if (seg_cell || seg_length) {
    if (int64_t(cells.size()) > seg_cap) return fail(ctx, DP_ERR_ARG, "segment arrays too small");
    if (seg_cell) std::copy(cells.begin(), cells.end(), seg_cell);
    if (seg_length) std::copy(lens.begin(), lens.end(), seg_length);
  }
  return DP_OK;
}

}  // extern "C"

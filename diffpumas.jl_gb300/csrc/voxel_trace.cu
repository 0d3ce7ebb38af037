// voxel_trace.cu -- directional paths through a voxel volume
// (examples/lvd_tomography.jl:583-627 voxel_cell_indices /
// distance_to_voxel_boundary, :738-779 trace_path(::VoxelVolume),
// :835-861 precompute_paths).  Host code: it runs once per geometry and
// produces the segment lists (cell, length) that the water-fraction CSDA
// model and the fixed-path MC consume.  FP64 with the reference's operations,
// so the segments are the reference's.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace {

constexpr double kPointEps = 1e-4;  // POINT_EPS (examples/lvd_tomography.jl:147)

// Julia searchsortedlast on sorted edges: the last index with e[i] <= x (0-based; -1 if none).
int last_le(const double* e, int n, double x) {
  return int(std::upper_bound(e, e + n, x) - e) - 1;
}

bool cell_of(const dp_voxel_volume& v, double x, double y, double z, int* i, int* j, int* k) {
  const int nx = v.nx + 1, ny = v.ny + 1, nz = v.nz + 1;  // edge counts
  if (x < v.x_edges[0] || x > v.x_edges[nx - 1] || y < v.y_edges[0] || y > v.y_edges[ny - 1] ||
      z < v.z_edges[0] || z > v.z_edges[nz - 1])
    return false;
  *i = std::min(std::max(last_le(v.x_edges, nx, x), 0), v.nx - 1);
  *j = std::min(std::max(last_le(v.y_edges, ny, y), 0), v.ny - 1);
  *k = std::min(std::max(last_le(v.z_edges, nz, z), 0), v.nz - 1);
  return true;
}

double to_boundary(const dp_voxel_volume& v, double x, double y, double z, double dx, double dy,
                   double dz) {
  int i, j, k;
  if (!cell_of(v, x, y, z, &i, &j, &k)) return 0.0;
  const double eps = 1e-10;
  double t_min = INFINITY;
  auto axis = [&](double d, double lo, double hi, double p) {
    if (std::fabs(d) > eps) {
      double t = d > 0 ? (hi - p) / d : (lo - p) / d;
      if (t > eps) t_min = std::min(t_min, t);
    }
  };
  axis(dx, v.x_edges[i], v.x_edges[i + 1], x);
  axis(dy, v.y_edges[j], v.y_edges[j + 1], y);
  axis(dz, v.z_edges[k], v.z_edges[k + 1], z);
  return std::isfinite(t_min) ? t_min : 0.0;
}

// trace_path(::VoxelVolume): the march from the detector (origin) along the
// direction until the surface exit at slant distance `surface`.
void trace(const dp_voxel_volume& v, double zenith, double azimuth, double surface,
           std::vector<int32_t>* cells, std::vector<double>* lens, double* traveled_out) {
  const double th = zenith * (M_PI / 180.0), ph = azimuth * (M_PI / 180.0);
  const double dh = std::sin(th);
  const double ux = dh * std::sin(ph), uy = dh * std::cos(ph), uz = std::cos(th);
  double x = ux * kPointEps, y = uy * kPointEps, z = uz * kPointEps;
  double traveled = kPointEps;
  for (long guard = 0; traveled < surface - kPointEps && guard < 100000000; ++guard) {
    int i, j, k;
    if (!cell_of(v, x, y, z, &i, &j, &k)) break;
    const int cell = i + v.nx * (j + v.ny * k);
    const double dist = to_boundary(v, x, y, z, ux, uy, uz);
    if (!std::isfinite(dist) || dist <= 0.0) break;
    const double remaining = surface - traveled;
    const double step = std::min(dist, remaining);
    if (step > 1e-8) {
      cells->push_back(cell);
      lens->push_back(step);
      traveled += step;
    }
    if (dist >= remaining - 1e-6) break;
    x += ux * (step + kPointEps);
    y += uy * (step + kPointEps);
    z += uz * (step + kPointEps);
  }
  *traveled_out = traveled;
}

bool check_volume(const dp_voxel_volume* v) {
  if (!v || v->nx < 1 || v->ny < 1 || v->nz < 1 || !v->x_edges || !v->y_edges || !v->z_edges)
    return false;
  auto sorted = [](const double* e, int n) {
    for (int i = 1; i <= n; ++i)
      if (!(e[i] > e[i - 1])) return false;
    return true;
  };
  return sorted(v->x_edges, v->nx) && sorted(v->y_edges, v->ny) && sorted(v->z_edges, v->nz);
}

}  // namespace

using dp::fail;

extern "C" {

int dp_voxel_trace(dp_ctx* ctx, const dp_voxel_volume* volume, long n_dirs, const double* zenith,
                   const double* azimuth, const double* surface_distance, int64_t* seg_ptr,
                   int32_t* seg_cell, double* seg_length, int64_t seg_cap, double* traveled,
                   double* remaining_rock) {
  if (!check_volume(volume)) return fail(ctx, DP_ERR_ARG, "voxel edges must be increasing");
  if (n_dirs < 0 || (n_dirs > 0 && (!zenith || !azimuth || !surface_distance || !seg_ptr)))
    return fail(ctx, DP_ERR_ARG, "bad direction arrays");
  std::vector<int32_t> cells;
  std::vector<double> lens;
  seg_ptr[0] = 0;
  for (long d = 0; d < n_dirs; ++d) {
    const double s = surface_distance[d];
    double tr = NAN;
    if (std::isfinite(s) && s > 0.0) trace(*volume, zenith[d], azimuth[d], s, &cells, &lens, &tr);
    seg_ptr[d + 1] = int64_t(cells.size());
    if (traveled) traveled[d] = tr;
    if (remaining_rock) remaining_rock[d] = std::isfinite(tr) ? std::max(0.0, s - tr) : NAN;
  }
  if (seg_cell || seg_length) {
    if (int64_t(cells.size()) > seg_cap) return fail(ctx, DP_ERR_ARG, "segment arrays too small");
    if (seg_cell) std::copy(cells.begin(), cells.end(), seg_cell);
    if (seg_length) std::copy(lens.begin(), lens.end(), seg_length);
  }
  return DP_OK;
}

}  // extern "C"

// tomo.cu -- voxel-density tomography forward model and its density adjoint.
//
// Paths.  The geometry does not depend on the densities, so rays are traced
// once into a device-resident CSR list of segments (cell, length) together with
// the CSC permutation that the J^T r gather uses (the reference likewise traces
// once: examples/diff_flux_cube.jl:489-557, examples/lvd_tomography.jl:835-861).
// The march replicates trace_cube_path (examples/diff_flux_cube.jl:194-366):
// position-based boundary stepping, candidates x, y, z with strict
// improvement, 1e-10 tolerance, 1 cm nudge, 1000-step cap; it runs in
// correctly rounded FP64 without contraction, so the segment lists equal the
// reference's.  A side-exit remainder (exit below the top face) becomes one
// more segment of length (zmax - z_exit)/max(|cos theta|, 0.01) whose density
// is rho[side_cell] or a fixed side density (diff_flux_cube.jl:417-444).
//
// Evaluation.  One warp per ray, one lane per energy node.  Per segment:
// X = R(E), E' = R^-1(X + rho L), weight *= S(E')/S(E) * exp(-L/(beta gamma
// c tau)); then the closed-form air column and the GCCLY flux; the per-ray
// flux is (1/N) sum_n 2 w_n f_n (compute_flux_from_segments, :374-470).
//  * FP64 kernel: the reference's per-segment operations (parity mode).
//  * Mixed kernel: per-segment work in FP32 -- the range is carried as a float
//    pair (the inversion stays accurate near E_min), energies come from the
//    node energy times exp of a small log offset, stopping powers and decay
//    exponents in FP32; the node flux integral is accumulated in FP64.
// Adjoint: a reverse sweep over the segment list carries
// lambda_k = d log(flux)/d E_k; d flux/d rho_k = flux lambda_k dE_k/dY_k L_k.
// Lanes are reduced per segment by a fixed shuffle tree: one Jacobian entry per
// segment.  J^T r = per-cell sums over the precomputed CSC permutation, each
// bucket ordered by entry index -- no floating-point atomics, bitwise
// reproducible.
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace dp {

struct GridDev {
  int nx, ny, nz;
  double x0, y0, z0, dx, dy, dz, xmax, ymax, zmax;
};

static GridDev grid_dev(const dp_grid& g) {
  return GridDev{g.nx, g.ny, g.nz, g.x0, g.y0, g.z0, g.dx, g.dy, g.dz,
                 g.x0 + g.nx * g.dx, g.y0 + g.ny * g.dy, g.z0 + g.nz * g.dz};
}

// examples/diff_flux_cube.jl:132-148 (get_cell_indices)
__device__ __forceinline__ bool cell_of(const GridDev& g, double x, double y, double z, int& i,
                                        int& j, int& k) {
  if (x < g.x0 || x > g.xmax || y < g.y0 || y > g.ymax || z < g.z0 || z > g.zmax) return false;
  i = min(max(int(floor(__ddiv_rn(__dsub_rn(x, g.x0), g.dx))) + 1, 1), g.nx);
  j = min(max(int(floor(__ddiv_rn(__dsub_rn(y, g.y0), g.dy))) + 1, 1), g.ny);
  k = min(max(int(floor(__ddiv_rn(__dsub_rn(z, g.z0), g.dz))) + 1, 1), g.nz);
  return true;
}

// examples/diff_flux_cube.jl:194-298 (distance_to_boundary)
__device__ __forceinline__ double to_boundary(const GridDev& g, double x, double y, double z,
                                              double ux, double uy, double uz, int i, int j,
                                              int k, bool& exiting) {
  const double eps = 1e-10;
  double tmin = CUDART_INF;
  exiting = false;
  if (fabs(ux) > eps) {
    double b = ux > 0 ? __dadd_rn(g.x0, __dmul_rn(double(i), g.dx))
                      : __dadd_rn(g.x0, __dmul_rn(double(i - 1), g.dx));
    double t = __ddiv_rn(__dsub_rn(b, x), ux);
    if (t > eps && t < tmin) {
      tmin = t;
      exiting = ux > 0 ? (i + 1 > g.nx) : (i - 1 < 1);
    }
  }
  if (fabs(uy) > eps) {
    double b = uy > 0 ? __dadd_rn(g.y0, __dmul_rn(double(j), g.dy))
                      : __dadd_rn(g.y0, __dmul_rn(double(j - 1), g.dy));
    double t = __ddiv_rn(__dsub_rn(b, y), uy);
    if (t > eps && t < tmin) {
      tmin = t;
      exiting = uy > 0 ? (j + 1 > g.ny) : (j - 1 < 1);
    }
  }
  if (fabs(uz) > eps) {
    double b = uz > 0 ? __dadd_rn(g.z0, __dmul_rn(double(k), g.dz))
                      : __dadd_rn(g.z0, __dmul_rn(double(k - 1), g.dz));
    double t = __ddiv_rn(__dsub_rn(b, z), uz);
    if (t > eps && t < tmin) {
      tmin = t;
      exiting = uz > 0 ? (k + 1 > g.nz) : (k - 1 < 1);
    }
  }
  if (tmin == CUDART_INF) exiting = true;
  return tmin;
}

// examples/diff_flux_cube.jl:304-366 (trace_cube_path).  Calls emit(s, cell,
// L) per segment; returns the segment count, or -1 past `cap`.
template <class Emit>
__device__ __forceinline__ int trace(const GridDev& g, const dp_ray& r, int cap, double* z_exit,
                                     Emit emit) {
  double x = r.ox, y = r.oy, z = r.oz;
  int ns = 0;
  *z_exit = z;
  for (int step = 0; step < 1000; ++step) {
    int i, j, k;
    if (!cell_of(g, x, y, z, i, j, k)) break;
    bool exiting;
    double d = to_boundary(g, x, y, z, r.ux, r.uy, r.uz, i, j, k, exiting);
    if (d <= 1e-10 || !isfinite(d)) {
      x = __dadd_rn(x, __dmul_rn(r.ux, 0.01));
      y = __dadd_rn(y, __dmul_rn(r.uy, 0.01));
      z = __dadd_rn(z, __dmul_rn(r.uz, 0.01));
      continue;
    }
    if (ns >= cap) return -1;
    emit(ns, (i - 1) + g.nx * ((j - 1) + g.ny * (k - 1)), d);
    ++ns;
    x = __dadd_rn(x, __dmul_rn(r.ux, d));
    y = __dadd_rn(y, __dmul_rn(r.uy, d));
    z = __dadd_rn(z, __dmul_rn(r.uz, d));
    *z_exit = z;
    if (exiting) break;
  }
  return ns;
}

// ============================================================ path building
// One thread per ray: segments into a fixed-capacity slot, count per ray.
__global__ void trace_kernel(GridDev g, const dp_ray* rays, long n_rays, int cap, int side_cell,
                             int32_t* slot_cell, double* slot_len, int64_t* counts,
                             float4* geom, int* err_flag) {
  long r = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (r >= n_rays) return;
  dp_ray ray = rays[r];
  {
    double cs = cos_theta_star(ray.cos_theta);
    geom[r] = make_float4(float(cs), float(pow(cs, 1.29)),
                          float(1.0 / fmax(fabs(ray.cos_theta), 0.01)), float(ray.cos_theta));
  }
  int32_t* sc = slot_cell + size_t(r) * cap;
  double* sl = slot_len + size_t(r) * cap;
  double z_exit;
  int ns = trace(g, ray, cap - 1, &z_exit, [&](int s, int cell, double L) {
    sc[s] = cell;
    sl[s] = L;
  });
  if (ns < 0) {
    atomicExch(err_flag, 2);
    counts[r] = 0;
    return;
  }
  if (z_exit < g.zmax - kEps64) {
    sc[ns] = side_cell;
    sl[ns] = (g.zmax - z_exit) / fmax(fabs(ray.cos_theta), 0.01);
    ++ns;
  }
  counts[r] = ns;
}

__global__ void compact_kernel(const int64_t* row_ptr, long n_rays, int cap,
                               const int32_t* slot_cell, const double* slot_len, int32_t* cell,
                               double* len, int32_t* row_of) {
  long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  long r = idx / cap;
  int s = int(idx - r * cap);
  if (r >= n_rays) return;
  int64_t b = row_ptr[r];
  if (s >= row_ptr[r + 1] - b) return;
  cell[b + s] = slot_cell[idx];
  len[b + s] = slot_len[idx];
  row_of[b + s] = int32_t(r);
}

// Exclusive scan of int64 (two levels; the second level walks any number of
// block totals serially in one block).  out[n] receives the total.
constexpr int kScan = 1024;
__global__ void __launch_bounds__(kScan) scan_blocks(const int64_t* in, int64_t* out, long n,
                                                     int64_t* totals) {
  __shared__ int64_t sh[kScan];
  long i = blockIdx.x * long(kScan) + threadIdx.x;
  int64_t v = i < n ? in[i] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kScan; o <<= 1) {
    int64_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = sh[threadIdx.x] - v;
  if (threadIdx.x == kScan - 1) totals[blockIdx.x] = sh[kScan - 1];
}
__global__ void __launch_bounds__(kScan) scan_totals(int64_t* totals, long nb, int64_t* grand) {
  __shared__ int64_t sh[kScan];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long b0 = 0; b0 < nb; b0 += kScan) {
    long i = b0 + threadIdx.x;
    int64_t v = i < nb ? totals[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScan; o <<= 1) {
      int64_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) totals[i] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == kScan - 1) carry += sh[kScan - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *grand = carry;
}
__global__ void scan_add(int64_t* out, long n, const int64_t* totals, const int64_t* grand) {
  long i = blockIdx.x * long(kScan) + threadIdx.x;
  if (i < n) out[i] += totals[blockIdx.x];
  if (i == n - 1) out[n] = *grand;
}

__global__ void hist_kernel(const int32_t* col, long nnz, int64_t* count) {
  long e = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (e < nnz && col[e] >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(&count[col[e]]), 1ull);
}
__global__ void place_kernel(const int32_t* col, long nnz, const int64_t* cptr, int32_t* cursor,
                             int32_t* perm) {
  long e = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (e >= nnz || col[e] < 0) return;
  int c = col[e];
  perm[cptr[c] + atomicAdd(&cursor[c], 1)] = int32_t(e);
}
// Buckets are ordered by entry index.  Small buckets (<= kSmallBucket): one
// thread, insertion sort.  Large ones (cells next to a detector collect one
// entry per ray of that detector) are listed and sorted by a block each.
constexpr int kSmallBucket = 32;
__global__ void sort_small_buckets_kernel(const int64_t* cptr, long ncell, int32_t* perm,
                                          int32_t* big, int32_t* n_big) {
  long c = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (c >= ncell) return;
  int64_t b = cptr[c], e = cptr[c + 1];
  if (e - b > kSmallBucket) {
    big[atomicAdd(n_big, 1)] = int32_t(c);
    return;
  }
  for (int64_t i = b + 1; i < e; ++i) {
    int32_t x = perm[i];
    int64_t j = i - 1;
    while (j >= b && perm[j] > x) {
      perm[j + 1] = perm[j];
      --j;
    }
    perm[j + 1] = x;
  }
}
// One block per large bucket: bitonic sort in shared memory (padded with
// INT_MAX to a power of two); buckets beyond the shared capacity are sorted
// by repeated odd-even merges of shared-memory-sized runs in global memory.
constexpr int kSortCap = 32768;  // entries (128 KB of dynamic shared memory)
__global__ void __launch_bounds__(1024) sort_big_buckets_kernel(const int64_t* cptr, int32_t* perm,
                                                                const int32_t* big,
                                                                const int32_t* n_big) {
  extern __shared__ int32_t sh[];
  for (int bi = blockIdx.x; bi < *n_big; bi += gridDim.x) {
    const int c = big[bi];
    const int64_t b = cptr[c];
    const int m = int(cptr[c + 1] - b);
    if (m <= kSortCap) {
      int p2 = 1;
      while (p2 < m) p2 <<= 1;
      for (int i = threadIdx.x; i < p2; i += blockDim.x) sh[i] = i < m ? perm[b + i] : 0x7fffffff;
      __syncthreads();
      for (int k = 2; k <= p2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int i = threadIdx.x; i < p2; i += blockDim.x) {
            int l = i ^ j;
            if (l > i) {
              bool up = (i & k) == 0;
              int32_t a = sh[i], d = sh[l];
              if ((a > d) == up) {
                sh[i] = d;
                sh[l] = a;
              }
            }
          }
          __syncthreads();
        }
      for (int i = threadIdx.x; i < m; i += blockDim.x) perm[b + i] = sh[i];
      __syncthreads();
    } else {
      // odd-even transposition over the bucket (rare: more than kSortCap
      // entries in one cell); bounded by m passes
      for (int pass = 0; pass < m; ++pass) {
        for (int i = 2 * threadIdx.x + (pass & 1); i + 1 < m; i += 2 * blockDim.x) {
          int32_t a = perm[b + i], d = perm[b + i + 1];
          if (a > d) {
            perm[b + i] = d;
            perm[b + i + 1] = a;
          }
        }
        __syncthreads();
      }
    }
  }
}
// prow[p] = row of the p-th bucketed entry.  Only the first cptr[ncell]
// positions of perm are filled (side-exit entries at a fixed density have no
// cell and are not bucketed).
__global__ void permute_rows_kernel(const int32_t* perm, const int32_t* row_of,
                                    const int64_t* n_bucketed, int32_t* prow) {
  long p = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (p < *n_bucketed) prow[p] = row_of[perm[p]];
}

// ============================================================ evaluation
// Per energy node start of the mixed kernel, shared by all rays: the range
// R(E0) as a float pair, S(E0), E0 and the node's interval on the grid.
struct NodeInit {
  float yh, yl, S0, E0;
  int i0;
  float coef, q, pad;
};

struct EvalP {
  TabView tab;
  const float* tab32;
  const float4* geom;
  const NodeInit* node0;
  const int32_t* order;
  int ld32;
  int rock, air, n_nodes, seg_cap;
  double H, mass, ctau, air_dexp, zmax, side_density;
  const double *nE, *nq, *nw;
  const double* rho;
  const dp_ray* rays;
  long n_rays;
  const int64_t* row_ptr;
  const int32_t* cell;
  const double* len;
  double* flux;
  double* jval64;
  float* jval32;
  int* err_flag;
  int wait_iters;  // polls of the table-staging wait
};

__device__ __forceinline__ double seg_density(const EvalP& P, int c) {
  return c >= 0 ? P.rho[c] : P.side_density;
}

// d log D / d Eavg, D = exp(-L/(beta gamma ctau)), beta = sqrt(max(1-1/g^2, 1e-12))
__device__ __forceinline__ double decay_log(double L, double Eavg, double mass, double ctau,
                                            double* dlog) {
  double g = 1.0 + Eavg / mass, b2 = 1.0 - 1.0 / (g * g);
  bool clamp = !(b2 > 1e-12);
  double b = sqrt(clamp ? 1e-12 : b2), bg = b * g;
  if (dlog) *dlog = L / (ctau * bg * bg) * (clamp ? b : 1.0 / b) / mass;
  return -L / (bg * ctau);
}
__device__ __forceinline__ double dlogS(const TabView& t, const double* E, const double* lE,
                                        const double* S, double e) {
  Dd s = interp_logE(t, E, lE, S, dd(e, 1.0 / e), dd(log(e), 1.0 / e), nullptr);
  return s.d / s.v;
}
__device__ __forceinline__ double range_slope(const TabView& t, const double* E, const double* lE,
                                              const double* R, double e) {
  return interp_logE(t, E, lE, R, dd(e, 1.0), dd(log(e), 1.0 / e), nullptr).d;
}
__device__ __forceinline__ double inv_slope(const double* R, const double* E, const double* lE,
                                            int n, double Y) {
  return inverse_range(R, E, lE, n, dd(Y, 1.0), nullptr).d;
}

enum { T_E = 0, T_LOGE, T_RS, T_RR, T_AS, T_AR, T_NCOL };
constexpr int kWarps = 4;

// ---------------------------------------------------------------- FP64 kernel
template <bool ADJ>
__global__ void __launch_bounds__(kWarps * 32) eval64_kernel(EvalP P) {
  extern __shared__ __align__(16) double smem[];
  __shared__ uint64_t mbar;
  const int ld = P.tab.ld, n = P.tab.n;
  const double* src[T_NCOL] = {P.tab.col(0, DP_COL_E),          P.tab.col(0, DP_COL_LOGE),
                               P.tab.col(P.rock, DP_COL_CSDA_S), P.tab.col(P.rock, DP_COL_CSDA_R),
                               P.tab.col(P.air, DP_COL_CSDA_S),  P.tab.col(P.air, DP_COL_CSDA_R)};
  if (!stage_columns(smem, src, T_NCOL, uint32_t(ld * sizeof(double)), &mbar, P.wait_iters)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    return;
  }
  const double *tE = smem + T_E * ld, *tlE = smem + T_LOGE * ld;
  const double *rS = smem + T_RS * ld, *rR = smem + T_RR * ld;
  const double *aS = smem + T_AS * ld, *aR = smem + T_AR * ld;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, cap = P.seg_cap;
  double* sL = smem + T_NCOL * ld + size_t(warp) * cap * 3;
  double* sD = sL + cap;
  double* sJ = sD + cap;
  const double Emax = tE[n - 1];
  for (long q = blockIdx.x * long(kWarps) + warp; q < P.n_rays; q += long(gridDim.x) * kWarps) {
    const long r = P.order[q];
    const int64_t off = P.row_ptr[r];
    const int nseg = int(P.row_ptr[r + 1] - off);
    for (int s = lane; s < nseg; s += 32) {
      sL[s] = P.len[off + s];
      sD[s] = seg_density(P, P.cell[off + s]);
      sJ[s] = 0.0;
    }
    __syncwarp();
    const double cosz = P.rays[r].cos_theta;
    const double cs_safe = fmax(fabs(cosz), 0.01);
    const double Lair = (P.H - P.zmax) / cs_safe;
    const double Gair = fmax((1.205 * 12e3 / cs_safe) * P.air_dexp, 0.0);
    const double cs = cos_theta_star(cosz), cs129 = pow(cs, 1.29);
    double fsum = 0.0;
    for (int base = 0; base < P.n_nodes; base += 32) {
      const int nd = base + lane;
      const bool active = nd < P.n_nodes;
      double E = active ? P.nE[nd] : 1.0, w = 1.0;
      bool ok = active;
      int kc = -1, hint = 0;
      double Eprev_c = 0.0;
      for (int s = 0; s < nseg && ok; ++s) {
        double X = interp_logE(P.tab, tE, tlE, rR, dd(E), dd(log(E)), nullptr).v;
        double Ek = inverse_range(rR, tE, tlE, n, dd(X + sL[s] * sD[s]), &hint).v;
        if (!(Ek < 1e12)) {
          ok = false;
          break;
        }
        if (kc < 0 && Ek >= Emax) {
          kc = s;
          Eprev_c = E;
        }
        double Si = interp_logE(P.tab, tE, tlE, rS, dd(E), dd(log(E)), nullptr).v;
        double Sf = interp_logE(P.tab, tE, tlE, rS, dd(Ek), dd(log(Ek)), nullptr).v;
        w = w * (Sf / Si);
        w = w * exp(decay_log(sL[s], (E + Ek) / 2.0, P.mass, P.ctau, nullptr));
        E = Ek;
      }
      double f = 0.0, EN = E, Ef = 0.0;
      if (ok) {
        double Xa = interp_logE(P.tab, tE, tlE, aR, dd(E), dd(log(E)), nullptr).v;
        Ef = inverse_range(aR, tE, tlE, n, dd(Xa + Gair), nullptr).v;
        double Sa0 = interp_logE(P.tab, tE, tlE, aS, dd(E), dd(log(E)), nullptr).v;
        double Sa1 = interp_logE(P.tab, tE, tlE, aS, dd(Ef), dd(log(Ef)), nullptr).v;
        w = w * (Sa1 / Sa0);
        w = w * exp(decay_log(Lair, (E + Ef) / 2.0, P.mass, P.ctau, nullptr));
        f = w * gccly_flux(cs, cs129, Ef, P.nq[nd], nullptr);
      }
      const double coef = ok ? 2.0 * P.nw[nd] / P.n_nodes : 0.0;
      fsum += coef * f;
      if (ADJ) {
        const bool live = coef != 0.0 && f != 0.0;
        double lam = 0.0;
        if (live) {
          double aA, dlogF;
          decay_log(Lair, (EN + Ef) / 2.0, P.mass, P.ctau, &aA);
          gccly_flux(cs, cs129, Ef, P.nq[nd], &dlogF);
          double dEf = inv_slope(aR, tE, tlE, n,
                                 interp_logE(P.tab, tE, tlE, aR, dd(EN), dd(log(EN)), nullptr).v + Gair) *
                       range_slope(P.tab, tE, tlE, aR, EN);
          lam = dlogS(P.tab, tE, tlE, rS, EN) - dlogS(P.tab, tE, tlE, aS, EN) + 0.5 * aA +
                dEf * (dlogS(P.tab, tE, tlE, aS, Ef) + 0.5 * aA + dlogF);
        }
        double Ek = EN;
        for (int s = nseg - 1; s >= 0; --s) {
          double v = 0.0, Ekm1 = 0.0;
          if (live) {
            const double L = sL[s];
            if (kc >= 0 && s > kc) {
              Ekm1 = Emax;
            } else if (s == kc) {
              Ekm1 = Eprev_c;
            } else {
              double Y = interp_logE(P.tab, tE, tlE, rR, dd(Ek), dd(log(Ek)), nullptr).v;
              Ekm1 = s == 0 ? P.nE[nd] : inverse_range(rR, tE, tlE, n, dd(Y - L * sD[s]), nullptr).v;
            }
            double Ycur = interp_logE(P.tab, tE, tlE, rR, dd(Ekm1), dd(log(Ekm1)), nullptr).v + L * sD[s];
            double Kp = (Ek >= Emax) ? 0.0 : inv_slope(rR, tE, tlE, n, Ycur);
            double a;
            decay_log(L, (Ekm1 + Ek) / 2.0, P.mass, P.ctau, &a);
            lam += 0.5 * a;
            v = coef * f * lam * Kp * L;
            lam = lam * Kp * range_slope(P.tab, tE, tlE, rR, Ekm1) + 0.5 * a;
          }
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if (lane == 0) sJ[s] += v;
          Ek = Ekm1;
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
    if (lane == 0) P.flux[r] = fsum;
    __syncwarp();
    if (ADJ)
      for (int s = lane; s < nseg; s += 32) P.jval64[off + s] = sJ[s];
    __syncwarp();
  }
}

// ---------------------------------------------------------------- mixed kernel
// Node start from the FP64 tables (each block computes all nodes once).
__device__ __forceinline__ void node_init(const EvalP& P, int k, const float* RH32, NodeInit* out) {
  const double E0 = P.nE[k];
  const Dd lE = dd(log(E0));
  const double *E = P.tab.col(0, DP_COL_E), *LE = P.tab.col(0, DP_COL_LOGE);
  const double X0 = interp_logE(P.tab, E, LE, P.tab.col(P.rock, DP_COL_CSDA_R), dd(E0), lE, nullptr).v;
  const double S0 = interp_logE(P.tab, E, LE, P.tab.col(P.rock, DP_COL_CSDA_S), dd(E0), lE, nullptr).v;
  NodeInit o;
  o.yh = float(X0);
  o.yl = float(X0 - double(o.yh));
  o.S0 = float(S0);
  o.E0 = float(E0);
  int n = P.tab.n, i = 0;
  {  // bisection on the single-precision range column
    int lo = 0, hi = n - 1;
    while (lo < hi - 1) {
      int mid = (lo + hi) >> 1;
      if (o.yh < RH32[mid]) hi = mid; else lo = mid;
    }
    i = lo;
  }
  o.i0 = i;
  o.coef = float(2.0 * P.nw[k] / P.n_nodes);
  o.q = float(P.nq[k]);
  o.pad = 0.0f;
  out[k] = o;
}

// flux_gccly in single precision; *dlog = d log(flux)/dK.
__device__ __forceinline__ float gccly32(float cs, float cs129, float K, float q, float* dlog) {
  float Emu = K + float(kMuonMass);
  float a = 3.64f / (Emu * cs129);
  float ec = 1.1f * Emu * cs;
  float rpi = 1.0f + ec / 115.0f, rK = 1.0f + ec / 850.0f;
  float h = 1.0f / rpi + 0.054f / rK;
  float cf = q < 0.0f ? float(1.0 / 2.2766) : (q > 0.0f ? float(1.2766 / 2.2766) : 1.0f);
  float f = powf(1.0f + a, -2.7f) * (1.4e3f * powf(Emu, -2.7f) * h * cf);
  if (dlog) {
    float dh = -(1.1f * cs / 115.0f) / (rpi * rpi) - 0.054f * (1.1f * cs / 850.0f) / (rK * rK);
    *dlog = 2.7f * a / (Emu * (1.0f + a)) - 2.7f / Emu + dh / h;
  }
  return f;
}

// Float-pair accumulation (TwoSum): (h, l) += x
__device__ __forceinline__ void ff_add(float& h, float& l, float x) {
  float s = h + x;
  float bb = s - h;
  float e = (h - (s - bb)) + (x - bb);
  h = s;
  l += e;
}

// Interval i with RH[i] <= Y < RH[i+1], moving from the current i.
__device__ __forceinline__ int walk(const float* RH, int n, float yh, int i) {
  while (i < n - 2 && !(yh < RH[i + 1])) ++i;
  while (i > 0 && yh < RH[i]) --i;
  return i;
}

template <bool ADJ>
__global__ void __launch_bounds__(kWarps * 32, 8) eval32_kernel(EvalP P) {
  extern __shared__ __align__(16) float fsm[];
  __shared__ uint64_t mbar;
  const int ld = P.ld32, n = P.tab.n;
  const float* base = P.tab32;
  const double* src[2 * kNC32];
  for (int c = 0; c < kNC32; ++c) {
    src[c] = reinterpret_cast<const double*>(base + (size_t(P.rock) * kNC32 + c) * ld);
    src[kNC32 + c] = reinterpret_cast<const double*>(base + (size_t(P.air) * kNC32 + c) * ld);
  }
  if (!stage_columns(reinterpret_cast<double*>(fsm), src, 2 * kNC32, uint32_t(ld * sizeof(float)),
                     &mbar, P.wait_iters)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    return;
  }
  const float* rk = fsm;                       // rock columns
  const float* ak = fsm + size_t(kNC32) * ld;  // air columns
  const float *RH = rk + C32_RH * ld, *RL = rk + C32_RL * ld, *SR = rk + C32_S * ld;
  const float *EE = rk + C32_E * ld, *SLO = rk + C32_SLOPE * ld, *DS = rk + C32_DSDLE * ld;
  const float *DLE = rk + C32_DLE * ld;
  const float *aRH = ak + C32_RH * ld, *aRL = ak + C32_RL * ld, *aS = ak + C32_S * ld;
  const float *aSLO = ak + C32_SLOPE * ld, *aDS = ak + C32_DSDLE * ld;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, cap = P.seg_cap;
  float* sG = fsm + size_t(2 * kNC32) * ld + size_t(warp) * cap * 3;  // grammage rho L
  float* sL = sG + cap;                                              // length L
  float* sJ = sL + cap;                                              // Jacobian accumulator
  NodeInit* snode = reinterpret_cast<NodeInit*>(fsm + size_t(2 * kNC32) * ld + size_t(kWarps) * cap * 3);
  for (int k = threadIdx.x; k < P.n_nodes; k += blockDim.x) node_init(P, k, RH, snode);
  __syncthreads();
  const float inv_m = float(1.0 / P.mass), inv_ctau = float(1.0 / P.ctau);
  const float Lair_c = float(P.H - P.zmax), Gair_c = float(1.205 * 12e3 * P.air_dexp);
  const float m_ctau = float(P.mass * P.ctau);
  const float Emax = EE[n - 1];
  for (long q = blockIdx.x * long(kWarps) + warp; q < P.n_rays; q += long(gridDim.x) * kWarps) {
    const long r = P.order[q];
    const int64_t off = P.row_ptr[r];
    const int nseg = int(P.row_ptr[r + 1] - off);
    for (int s = lane; s < nseg; s += 32) {
      const float L = float(P.len[off + s]);
      sG[s] = L * float(seg_density(P, P.cell[off + s]));
      sL[s] = L;
      sJ[s] = 0.0f;
    }
    __syncwarp();
    const float4 gm = P.geom[r];
    const float cs = gm.x, cs129 = gm.y, inv_cs = gm.z;
    const float Lair = Lair_c * inv_cs;
    const float Gh = fmaxf(Gair_c * inv_cs, 0.0f), Gl = 0.0f;
    double fsum = 0.0;
    for (int b0 = 0; b0 < P.n_nodes; b0 += 32) {
      const int nd = b0 + lane;
      const bool active = nd < P.n_nodes;
      const NodeInit ni = snode[active ? nd : 0];
      const float S0 = ni.S0, E0 = ni.E0;
      float yh = ni.yh, yl = ni.yl;
      const int i0 = ni.i0;
      int i = i0;
      float Eprev = E0, E = E0, u = 0.0f, dsum = 0.0f;
      bool clamped = false;
      for (int s = 0; s < nseg; ++s) {
        ff_add(yh, yl, sG[s]);
        i = walk(RH, n, yh, i);
        clamped = !(yh < RH[n - 1]);
        u = clamped ? DLE[n - 2] : fminf(((yh - RH[i]) + (yl - RL[i])) * SLO[i], DLE[i]);
        if (clamped) i = n - 2;
        E = clamped ? Emax : EE[i] * __expf(u);
        float x = 0.5f * (Eprev + E) * inv_m;
        dsum -= sL[s] * rsqrtf(x * (x + 2.0f));
        Eprev = E;
      }
      const float EN = E, uN = u;
      const int iN = i;
      const bool clampN = clamped;
      const float SN = SR[iN] + uN * DS[iN];
      // air column: R_air(E_N) on the same energy interval, + closed-form grammage
      float ah = aRH[iN], al = aRL[iN];
      ff_add(ah, al, uN / aSLO[iN]);
      ff_add(ah, al, Gh);
      al += Gl;
      int j = walk(aRH, n, ah, iN);
      const bool clampF = !(ah < aRH[n - 1]);
      const float ua = clampF ? DLE[n - 2] : fminf(((ah - aRH[j]) + (al - aRL[j])) * aSLO[j], DLE[j]);
      if (clampF) j = n - 2;
      const float Ef = clampF ? Emax : EE[j] * __expf(ua);
      const float SaN = aS[iN] + uN * aDS[iN], SaF = aS[j] + ua * aDS[j];
      const float xa = 0.5f * (EN + Ef) * inv_m;
      const float ibga = rsqrtf(xa * (xa + 2.0f));
      const float w = (SN / S0) * (SaF / SaN) * __expf((dsum - Lair * ibga) * inv_ctau);
      float dlogF = 0.0f;
      const float F = gccly32(cs, cs129, Ef, ni.q, ADJ ? &dlogF : nullptr);
      const float f = active ? w * F : 0.0f;
      const float coef = active ? ni.coef : 0.0f;
      fsum += double(coef) * double(f);  // node integral accumulated in FP64
      if (ADJ) {
        const float cf = coef * f;
        float lam = 0.0f;
        if (cf != 0.0f) {
          const float aA = Lair * (xa + 1.0f) * ibga * ibga * ibga / m_ctau;
          const float dEf = (clampF || clampN) ? 0.0f : (Ef * aSLO[j]) / (EN * aSLO[iN]);
          const float dSr = clampN ? 0.0f : DS[iN] / (SN * EN);
          const float dSaN = clampN ? 0.0f : aDS[iN] / (SaN * EN);
          const float dSaF = clampF ? 0.0f : aDS[j] / (SaF * Ef);
          lam = dSr - dSaN + 0.5f * aA + dEf * (dSaF + 0.5f * aA + dlogF);
        }
        float Ek = EN;
        int ik = iN;
        bool ck = clampN;
        for (int s = nseg - 1; s >= 0; --s) {
          // previous point E_{k-1}
          ff_add(yh, yl, -sG[s]);
          float Ekm1;
          int im;
          if (s == 0) {
            Ekm1 = E0;
            im = i0;
          } else {
            im = walk(RH, n, yh, ik);
            float um = fminf(fmaxf(((yh - RH[im]) + (yl - RL[im])) * SLO[im], 0.0f), DLE[im]);
            Ekm1 = EE[im] * __expf(um);
            if (!(yh < RH[n - 1])) {
              Ekm1 = Emax;
              im = n - 2;
            }
          }
          const bool cm = !(Ekm1 < Emax);
          const float Kp = ck ? 0.0f : Ek * SLO[ik];
          const float x = 0.5f * (Ekm1 + Ek) * inv_m;
          const float ib = rsqrtf(x * (x + 2.0f));
          const float a = sL[s] * (x + 1.0f) * ib * ib * ib / m_ctau;
          lam += 0.5f * a;
          float v = cf * lam * Kp * sL[s];
          const float Rp = cm ? 0.0f : 1.0f / (Ekm1 * SLO[im]);
          lam = lam * Kp * Rp + 0.5f * a;
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if (lane == 0) sJ[s] += v;
          Ek = Ekm1;
          ik = im;
          ck = cm;
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
    if (lane == 0) P.flux[r] = fsum;
    __syncwarp();
    if (ADJ)
      for (int s = lane; s < nseg; s += 32) P.jval32[off + s] = sJ[s];
    __syncwarp();
  }
}

// J^T r over the precomputed CSC permutation of a large bucket: one block of
// kBigThreads per cell; thread t sums entries t, t + kBigThreads, ... in
// order, then big_block_sum -- the same arithmetic order on every call.
// perm == nullptr: the values are already in CSC order.
template <class V>
__global__ void __launch_bounds__(kBigThreads) gather_big_kernel(
    const int64_t* cptr, const int32_t* perm, const V* val, const int32_t* prow,
    const double* cot, const int32_t* big, int n_big, double* grad) {
  __shared__ double sh[kBigThreads / 32];
  const int c = big[blockIdx.x];
  double s = 0.0;
  for (int64_t p = cptr[c] + threadIdx.x, e = cptr[c + 1]; p < e; p += kBigThreads)
    s += double(val[perm ? perm[p] : p]) * cot[prow[p]];
  s = big_block_sum(s, sh);
  if (threadIdx.x == 0) grad[c] = s;
}
// Cells with at most kSmallBucket entries: one thread, entries in order.
template <class V>
__global__ void gather_small_kernel(const int64_t* cptr, const int32_t* perm, const V* val,
                                    const int32_t* prow, const double* cot, long ncell,
                                    double* grad) {
  long c = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (c >= ncell) return;
  int64_t b = cptr[c], e = cptr[c + 1];
  if (e - b > kSmallBucket) return;  // gather_big_kernel
  double s = 0.0;
  for (int64_t p = b; p < e; ++p) s += double(val[perm ? perm[p] : p]) * cot[prow[p]];
  grad[c] = s;
}
// The Jacobian values of the bucketed entries in CSC order (out[p] =
// val[perm[p]] for p < *n_bucketed), so that repeated J^T v products read
// them contiguously.
template <class V>
__global__ void csc_values_kernel(const int32_t* perm, const V* val, const int64_t* n_bucketed,
                                  int64_t n, V* out) {
  const int64_t m = *n_bucketed;
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < m && p < n;
       p += int64_t(gridDim.x) * blockDim.x)
    out[p] = val[perm[p]];
}

// ---------------------------------------------------------------- plain form
// Plain FP64 form: one launch per ray, one thread per node, global tables,
// bisection lookups, no staging, the ray traced by every thread.
__global__ void plain_ray_kernel(EvalP P, GridDev g, int side_cell, long r, double* part) {
  int nd = threadIdx.x;
  if (nd >= P.n_nodes) return;
  const TabView& t = P.tab;
  const double *E_ = t.col(0, DP_COL_E), *lE = t.col(0, DP_COL_LOGE);
  const double *rS = t.col(P.rock, DP_COL_CSDA_S), *rR = t.col(P.rock, DP_COL_CSDA_R);
  const double *aS = t.col(P.air, DP_COL_CSDA_S), *aR = t.col(P.air, DP_COL_CSDA_R);
  TabView tb = t;
  tb.uniform = 0;
  dp_ray ray = P.rays[r];
  double E = P.nE[nd], w = 1.0;
  bool ok = true;
  double z_exit;
  auto seg = [&](double rho, double L) {
    if (!ok) return;
    double X = interp_logE(tb, E_, lE, rR, dd(E), dd(log(E)), nullptr).v;
    double Ek = inverse_range(rR, E_, lE, t.n, dd(X + L * rho), nullptr).v;
    if (!(Ek < 1e12)) {
      ok = false;
      return;
    }
    w *= interp_logE(tb, E_, lE, rS, dd(Ek), dd(log(Ek)), nullptr).v /
         interp_logE(tb, E_, lE, rS, dd(E), dd(log(E)), nullptr).v;
    w *= exp(decay_log(L, (E + Ek) / 2.0, P.mass, P.ctau, nullptr));
    E = Ek;
  };
  trace(g, ray, 1 << 30, &z_exit, [&](int, int cell, double L) { seg(P.rho[cell], L); });
  double cs_safe = fmax(fabs(ray.cos_theta), 0.01);
  if (z_exit < g.zmax - kEps64)
    seg(side_cell >= 0 ? P.rho[side_cell] : P.side_density, (g.zmax - z_exit) / cs_safe);
  double f = 0.0;
  if (ok) {
    double Xa = interp_logE(tb, E_, lE, aR, dd(E), dd(log(E)), nullptr).v;
    double Gair = fmax((1.205 * 12e3 / cs_safe) * P.air_dexp, 0.0);
    double Ef = inverse_range(aR, E_, lE, t.n, dd(Xa + Gair), nullptr).v;
    w *= interp_logE(tb, E_, lE, aS, dd(Ef), dd(log(Ef)), nullptr).v /
         interp_logE(tb, E_, lE, aS, dd(E), dd(log(E)), nullptr).v;
    w *= exp(decay_log((P.H - g.zmax) / cs_safe, (E + Ef) / 2.0, P.mass, P.ctau, nullptr));
    double cs = cos_theta_star(ray.cos_theta);
    f = w * gccly_flux(cs, pow(cs, 1.29), Ef, P.nq[nd], nullptr);
  }
  part[r * P.n_nodes + nd] = 2.0 * P.nw[nd] * f / P.n_nodes;
}
__global__ void plain_sum_kernel(const double* v, long n_rays, int n_nodes, double* flux) {
  long r = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (r >= n_rays) return;
  double s = 0.0;
  for (int k = 0; k < n_nodes; ++k) s += v[r * n_nodes + k];
  flux[r] = s;
}

// ============================================================ host side
static int check(dp_ctx* ctx) {
  if (!ctx->blocking) return DP_OK;  // deferred to dp_sync
  int flag = 0;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return fail(ctx, DP_ERR_STATE,
                flag == 2 ? "ray segment buffer overflow" : "table-staging wait exceeded its limit");
  }
  return DP_OK;
}

static void launch_scan(dp_ctx* ctx, const int64_t* in, int64_t* out, long n, int64_t* totals) {
  long nb = (n + kScan - 1) / kScan;
  if (nb < 1) nb = 1;
  scan_blocks<<<int(nb), kScan, 0, ctx->stream>>>(in, out, n, totals);
  scan_totals<<<1, kScan, 0, ctx->stream>>>(totals, nb, totals + nb + 1);
  scan_add<<<int(nb), kScan, 0, ctx->stream>>>(out, n, totals, totals + nb + 1);
  ctx->launches += 3;
}

template <class T>
static T* dalloc(std::vector<void*>& keep, size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
  keep.push_back(p);
  return static_cast<T*>(p);
}

static void free_paths_arrays(dp_paths* p) {
  if (!p->owned) return;
  for (void* x : {(void*)p->rays, (void*)p->row_ptr, (void*)p->cell, (void*)p->len,
                  (void*)p->row_of, (void*)p->cptr, (void*)p->perm, (void*)p->geom,
                  (void*)p->order, (void*)p->prow, (void*)p->big})
    if (x) cudaFree(x);
}

// Builds the paths handle from device rays.  Temporaries live in scratch slot
// 3.  With `arena` the handle's arrays are carved from that arena too (a
// one-shot handle, not owned); otherwise they are cudaMalloc'ed (owned).
static int build_paths(dp_ctx* ctx, const dp_grid& gr, const dp_ray* d_rays_in, long n_rays,
                       int side_cell, bool copy_rays, dp_paths** out, Arena* arena = nullptr) {
  long ncell = long(gr.nx) * gr.ny * gr.nz;
  const int cap = std::min(1001, gr.nx + gr.ny + gr.nz + 64) + 1;
  long nbr = (n_rays + kScan) / kScan + 1;
  long nbc = (ncell + kScan) / kScan + 1;
  dp_paths* P = new dp_paths;
  P->ctx = ctx;
  P->device = ctx->device;
  P->grid = gr;
  P->side_cell = side_cell;
  P->n_rays = n_rays;
  P->owned = arena == nullptr;
  // temporaries: slot arrays, counts, scan totals, cell histogram, cursors
  size_t tbytes = size_t(n_rays) * cap * 12 + size_t(n_rays + nbr + 4) * 8 +
                  size_t(ncell + 1) * 16 + size_t(nbc + 2) * 8 + 24 * 256;
  Arena tmp;
  if (!arena) {
    tmp.base = static_cast<char*>(scratch(ctx, tbytes, 3));
    tmp.cap = ctx->slot_bytes[3];
  }
  Arena& T = arena ? *arena : tmp;
  auto bail = [&](int code, const char* msg) {
    free_paths_arrays(P);
    delete P;
    return fail(ctx, code, msg);
  };
  auto perm_alloc = [&](size_t bytes) -> void* {
    if (arena) return arena->take<char>(bytes);
    void* p = nullptr;
    return cudaMalloc(&p, bytes ? bytes : 1) == cudaSuccess ? p : nullptr;
  };
  if (copy_rays) {
    P->rays = static_cast<dp_ray*>(perm_alloc(sizeof(dp_ray) * n_rays));
    if (!P->rays) return bail(DP_ERR_ALLOC, "device allocation failed");
    if (cudaMemcpyAsync(P->rays, d_rays_in, sizeof(dp_ray) * n_rays, cudaMemcpyDeviceToDevice,
                        ctx->stream) != cudaSuccess)
      return bail(DP_ERR_CUDA, "ray copy failed");
  }
  const dp_ray* rays = copy_rays ? P->rays : d_rays_in;
  P->row_ptr = static_cast<int64_t*>(perm_alloc(sizeof(int64_t) * (n_rays + 1)));
  P->geom = static_cast<float4*>(perm_alloc(sizeof(float4) * n_rays));
  int32_t* slot_cell = T.take<int32_t>(size_t(n_rays) * cap);
  double* slot_len = T.take<double>(size_t(n_rays) * cap);
  int64_t* counts = T.take<int64_t>(n_rays + 1);
  int64_t* totals = T.take<int64_t>(nbr + 2);
  if (!P->row_ptr || !P->geom || !slot_cell || !slot_len || !counts || !totals)
    return bail(DP_ERR_ALLOC, "device allocation failed");
  GridDev g = grid_dev(gr);
  timed_begin(ctx);
  // 32 rays per block: the serial FP64 march spreads over all SMs
  trace_kernel<<<int((n_rays + 31) / 32), 32, 0, ctx->stream>>>(g, rays, n_rays, cap, side_cell,
                                                                     slot_cell, slot_len, counts,
                                                                     P->geom, ctx->d_flag);
  timed_end(ctx, "tomo_trace");
  launch_scan(ctx, counts, P->row_ptr, n_rays, totals);
  int64_t nnz = 0;
  if (cudaMemcpyAsync(&nnz, P->row_ptr + n_rays, 8, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return bail(DP_ERR_CUDA, "copy failed");
  int rc = dp_sync(ctx);
  if (rc) {
    std::string m = ctx->err;
    return bail(rc, m.c_str());
  }
  // longest list
  std::vector<int64_t> hc(n_rays);
  cudaMemcpy(hc.data(), counts, 8 * n_rays, cudaMemcpyDeviceToHost);
  int mx = 0;
  for (long r = 0; r < n_rays; ++r) mx = std::max<int>(mx, int(hc[r]));
  P->nnz = nnz;
  P->max_seg = mx;
  P->cell = static_cast<int32_t*>(perm_alloc(sizeof(int32_t) * (nnz + 1)));
  P->len = static_cast<double*>(perm_alloc(sizeof(double) * (nnz + 1)));
  P->row_of = static_cast<int32_t*>(perm_alloc(sizeof(int32_t) * (nnz + 1)));
  P->cptr = static_cast<int64_t*>(perm_alloc(sizeof(int64_t) * (ncell + 1)));
  P->perm = static_cast<int32_t*>(perm_alloc(sizeof(int32_t) * (nnz + 1)));
  if (!P->cell || !P->len || !P->row_of || !P->cptr || !P->perm)
    return bail(DP_ERR_ALLOC, "device allocation failed");
  long tot = n_rays * long(cap);
  compact_kernel<<<int((tot + 255) / 256), 256, 0, ctx->stream>>>(P->row_ptr, n_rays, cap, slot_cell,
                                                                   slot_len, P->cell, P->len, P->row_of);
  ++ctx->launches;
  // CSC permutation (entries of the side remainder at a fixed density excluded)
  int64_t* ccount = T.take<int64_t>(ncell + 1);
  int32_t* cursor = T.take<int32_t>(ncell + 1);
  int64_t* ctot = T.take<int64_t>(nbc + 2);
  if (!ccount || !cursor || !ctot) return bail(DP_ERR_ALLOC, "device allocation failed");
  cudaMemsetAsync(ccount, 0, 8 * (ncell + 1), ctx->stream);
  cudaMemsetAsync(cursor, 0, 4 * (ncell + 1), ctx->stream);
  if (nnz > 0) hist_kernel<<<int((nnz + 255) / 256), 256, 0, ctx->stream>>>(P->cell, nnz, ccount);
  launch_scan(ctx, ccount, P->cptr, ncell, ctot);
  if (nnz > 0) place_kernel<<<int((nnz + 255) / 256), 256, 0, ctx->stream>>>(P->cell, nnz, P->cptr, cursor, P->perm);
  int32_t* big = T.take<int32_t>(ncell + 1);
  int32_t* n_big = T.take<int32_t>(1);
  P->prow = static_cast<int32_t*>(perm_alloc(sizeof(int32_t) * (nnz + 1)));
  P->order = static_cast<int32_t*>(perm_alloc(sizeof(int32_t) * (n_rays + 1)));
  if (!big || !n_big || !P->prow || !P->order) return bail(DP_ERR_ALLOC, "device allocation failed");
  cudaMemsetAsync(n_big, 0, 4, ctx->stream);
  sort_small_buckets_kernel<<<int((ncell + 255) / 256), 256, 0, ctx->stream>>>(P->cptr, ncell, P->perm,
                                                                               big, n_big);
  cudaFuncSetAttribute(sort_big_buckets_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kSortCap * 4);
  sort_big_buckets_kernel<<<152, 1024, kSortCap * 4, ctx->stream>>>(P->cptr, P->perm, big, n_big);
  if (nnz > 0)
    permute_rows_kernel<<<int((nnz + 255) / 256), 256, 0, ctx->stream>>>(P->perm, P->row_of,
                                                                          P->cptr + ncell, P->prow);
  ctx->launches += 5;
  // schedule: longest ray first (stable), so that the tail of the launch is short
  {
    std::vector<int32_t> ord(n_rays);
    for (long r = 0; r < n_rays; ++r) ord[r] = int32_t(r);
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return hc[a] > hc[b]; });
    if (cudaMemcpyAsync(P->order, ord.data(), 4 * n_rays, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(&P->n_big, n_big, 4, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      return bail(DP_ERR_CUDA, "schedule upload failed");
    // the large-bucket list survives the build (the temporaries do not)
    int32_t* keep = static_cast<int32_t*>(perm_alloc(sizeof(int32_t) * (P->n_big + 1)));
    if (!keep) return bail(DP_ERR_ALLOC, "device allocation failed");
    if (P->n_big > 0)
      cudaMemcpyAsync(keep, big, 4 * size_t(P->n_big), cudaMemcpyDeviceToDevice, ctx->stream);
    P->big = keep;
  }
  if (cudaGetLastError() != cudaSuccess) return bail(DP_ERR_CUDA, "path build launch failed");
  rc = check(ctx);
  if (rc) {
    free_paths_arrays(P);
    delete P;
    return rc;
  }
  *out = P;
  return DP_OK;
}

static int make_eval(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa, const dp_tomo_params* tp,
                     EvalP& P) {
  if (!ctx || !ph || !pa || !tp) return fail(ctx, DP_ERR_ARG, "null argument");
  if (tp->n_nodes <= 0 || !tp->node_energy || !tp->node_charge || !tp->node_weight)
    return fail(ctx, DP_ERR_ARG, "energy nodes required");
  if (tp->rock_material < 0 || tp->rock_material >= ph->n_mat || tp->air_material < 0 ||
      tp->air_material >= ph->n_mat)
    return fail(ctx, DP_ERR_ARG, "material index out of range");
  P = EvalP{};
  P.tab = ph->view;
  P.tab32 = ph->dev32;
  P.ld32 = ph->ld32;
  P.rock = tp->rock_material;
  P.air = tp->air_material;
  P.n_nodes = tp->n_nodes;
  P.seg_cap = std::max(pa->max_seg, 1);
  P.H = tp->primary_altitude > 0 ? tp->primary_altitude : 3e4;
  P.mass = ph->settings.mass;
  P.ctau = ph->settings.ctau;
  P.zmax = pa->grid.z0 + pa->grid.nz * pa->grid.dz;
  P.air_dexp = std::exp(-P.zmax / 12e3) - std::exp(-P.H / 12e3);
  P.side_density = tp->side_density;
  P.rays = pa->rays;
  P.geom = pa->geom;
  P.order = pa->order;
  P.n_rays = pa->n_rays;
  P.row_ptr = pa->row_ptr;
  P.cell = pa->cell;
  P.len = pa->len;
  P.err_flag = ctx->d_flag;
  P.wait_iters = stage_wait(ctx);
  return DP_OK;
}

// Core evaluation on device pointers.  precision: 0 = FP64, 1 = mixed.
__global__ void widen_kernel(const float* in, int64_t n, double* out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = double(in[i]);
}

static int eval_core(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa, const dp_tomo_params* tp,
                     const double* rho, const double* nE, const double* nq, const double* nw,
                     const double* cot, double* flux, double* grad, double* jac, int precision,
                     void* jraw = nullptr) {
  EvalP P;
  int rc = make_eval(ctx, ph, pa, tp, P);
  if (rc) return rc;
  if (pa->n_rays == 0) return DP_OK;
  P.rho = rho;
  P.nE = nE;
  P.nq = nq;
  P.nw = nw;
  P.flux = flux;
  const bool adj = (cot && grad) || jac || jraw;
  // slot 1: node starts, then the Jacobian values
  size_t need = size_t(P.n_nodes) * sizeof(NodeInit) + size_t(pa->nnz + 1) * 8 + 1024;
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, need, 1));
  A.cap = ctx->slot_bytes[1];
  if (!A.base) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  void* jbuf = nullptr;
  if (adj) {
    jbuf = jraw ? jraw
                : jac && !precision ? (void*)jac
                                    : A.take<char>(size_t(pa->nnz + 1) * (precision ? 4 : 8));
    if (!jbuf) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  }
  long blocks = std::min<long>((pa->n_rays + kWarps - 1) / kWarps, 152L * 16);
  size_t smem;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(eval64_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    cudaFuncSetAttribute(eval64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    cudaFuncSetAttribute(eval32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    cudaFuncSetAttribute(eval32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr = true;
  }
  timed_begin(ctx);
  if (precision == 0) {
    smem = size_t(T_NCOL) * P.tab.ld * 8 + size_t(kWarps) * P.seg_cap * 3 * 8;
    if (smem > 220 * 1024) return fail(ctx, DP_ERR_ARG, "ray too long for the FP64 kernel");
    P.jval64 = static_cast<double*>(jbuf);
    if (adj) eval64_kernel<true><<<int(blocks), kWarps * 32, smem, ctx->stream>>>(P);
    else eval64_kernel<false><<<int(blocks), kWarps * 32, smem, ctx->stream>>>(P);
  } else {
    smem = size_t(2 * kNC32) * P.ld32 * 4 + size_t(kWarps) * P.seg_cap * 3 * 4 +
           size_t(P.n_nodes) * sizeof(NodeInit);
    if (smem > 220 * 1024) return fail(ctx, DP_ERR_ARG, "ray too long for the mixed kernel");
    P.jval32 = static_cast<float*>(jbuf);
    if (adj) eval32_kernel<true><<<int(blocks), kWarps * 32, smem, ctx->stream>>>(P);
    else eval32_kernel<false><<<int(blocks), kWarps * 32, smem, ctx->stream>>>(P);
  }
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, adj ? "tomo_adjoint" : "tomo_forward");
  if (adj && cot && grad) {
    int rc2 = tomo_transpose(ctx, pa, jbuf, precision, cot, grad);
    if (rc2) return rc2;
  }
  if (jac && precision) {
    widen_kernel<<<int(std::min<long>((pa->nnz + 255) / 256, 152L * 64)), 256, 0, ctx->stream>>>(
        static_cast<const float*>(jbuf), pa->nnz, jac);
    ++ctx->launches;
    DP_CHECK_CUDA(ctx, cudaGetLastError());
  }
  return ctx->blocking ? check(ctx) : DP_OK;
}

int tomo_csc_values(dp_ctx* ctx, const dp_paths* pa, const void* jbuf, int precision,
                    void* out) {
  const long ncell = long(pa->grid.nx) * pa->grid.ny * pa->grid.nz;
  const int blocks = int(std::min<int64_t>((pa->nnz + 255) / 256, 152L * 32));
  if (blocks < 1) return DP_OK;
  timed_begin(ctx);
  if (precision == 0)
    csc_values_kernel<double><<<blocks, 256, 0, ctx->stream>>>(
        pa->perm, static_cast<const double*>(jbuf), pa->cptr + ncell, pa->nnz,
        static_cast<double*>(out));
  else
    csc_values_kernel<float><<<blocks, 256, 0, ctx->stream>>>(
        pa->perm, static_cast<const float*>(jbuf), pa->cptr + ncell, pa->nnz,
        static_cast<float*>(out));
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "tomo_csc_values");
  return DP_OK;
}

// J^T v over the CSC buckets (deterministic segmented sums, no float atomics);
// csc: jbuf holds the values in CSC order (tomo_csc_values).
int tomo_transpose(dp_ctx* ctx, const dp_paths* pa, const void* jbuf, int precision,
                   const double* cot, double* grad, bool csc) {
  long ncell = long(pa->grid.nx) * pa->grid.ny * pa->grid.nz;
  const int32_t* perm = csc ? nullptr : pa->perm;
  {
    timed_begin(ctx);
    if (precision == 0) {
      const double* v = static_cast<const double*>(jbuf);
      gather_small_kernel<double><<<int((ncell + 255) / 256), 256, 0, ctx->stream>>>(
          pa->cptr, perm, v, pa->prow, cot, ncell, grad);
      if (pa->n_big > 0)
        gather_big_kernel<double><<<pa->n_big, kBigThreads, 0, ctx->stream>>>(
            pa->cptr, perm, v, pa->prow, cot, pa->big, pa->n_big, grad);
    } else {
      const float* v = static_cast<const float*>(jbuf);
      gather_small_kernel<float><<<int((ncell + 255) / 256), 256, 0, ctx->stream>>>(
          pa->cptr, perm, v, pa->prow, cot, ncell, grad);
      if (pa->n_big > 0)
        gather_big_kernel<float><<<pa->n_big, kBigThreads, 0, ctx->stream>>>(
            pa->cptr, perm, v, pa->prow, cot, pa->big, pa->n_big, grad);
    }
    ctx->launches += pa->n_big > 0 ? 1 : 0;
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "tomo_transpose");
  }
  return DP_OK;
}

// Flux, and the Jacobian values of the resident paths into jraw (FP32 for the
// mixed-precision kernel, FP64 otherwise); node arrays of tp on the device.
int tomo_eval_raw(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa, const dp_tomo_params* tp,
                  const double* rho, double* flux, void* jraw, int precision) {
  return eval_core(ctx, ph, pa, tp, rho, tp->node_energy, tp->node_charge, tp->node_weight,
                   nullptr, flux, nullptr, nullptr, precision, jraw);
}

}  // namespace dp

using namespace dp;

namespace {
// Device copies of host inputs carved from scratch slot 2 (reused across calls).
struct Inputs {
  double *rho = nullptr, *nE = nullptr, *nq = nullptr, *nw = nullptr, *flux = nullptr,
         *cot = nullptr, *grad = nullptr;
  dp_ray* rays = nullptr;
};
int upload_inputs(dp_ctx* ctx, const dp_tomo_params* tp, long ncell, long n_rays,
                  const dp_ray* rays, const double* rho, const double* cot, bool grad, Inputs& d) {
  size_t need = sizeof(dp_ray) * n_rays + 8 * (ncell * 2 + n_rays * 2 + 3 * tp->n_nodes) + 16 * 256;
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, need, 2));
  A.cap = ctx->slot_bytes[2];
  if (!A.base) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  d.rho = A.take<double>(ncell);
  d.nE = A.take<double>(tp->n_nodes);
  d.nq = A.take<double>(tp->n_nodes);
  d.nw = A.take<double>(tp->n_nodes);
  d.flux = A.take<double>(n_rays);
  if (rays) d.rays = A.take<dp_ray>(n_rays);
  if (cot) d.cot = A.take<double>(n_rays);
  if (grad) d.grad = A.take<double>(ncell);
  auto up = [&](void* dst, const void* src, size_t b) {
    return cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, ctx->stream) == cudaSuccess;
  };
  bool ok = up(d.rho, rho, 8 * ncell) && up(d.nE, tp->node_energy, 8 * tp->n_nodes) &&
            up(d.nq, tp->node_charge, 8 * tp->n_nodes) && up(d.nw, tp->node_weight, 8 * tp->n_nodes) &&
            (!rays || up(d.rays, rays, sizeof(dp_ray) * n_rays)) && (!cot || up(d.cot, cot, 8 * n_rays));
  return ok ? DP_OK : fail(ctx, DP_ERR_CUDA, "input upload failed");
}

int host_eval(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
              const double* rho, long n_rays, const dp_ray* rays, const double* cot, double* flux,
              double* grad, int64_t* row_ptr, int32_t* col, double* val, int64_t nnz_cap,
              int64_t* nnz, int precision) {
  if (!ctx || !ph || !gr || !tp) return fail(ctx, DP_ERR_ARG, "null argument");
  if (gr->nx <= 0 || gr->ny <= 0 || gr->nz <= 0 || !(gr->dx > 0) || !(gr->dy > 0) || !(gr->dz > 0))
    return fail(ctx, DP_ERR_ARG, "invalid grid");
  long ncell = long(gr->nx) * gr->ny * gr->nz;
  if (tp->side_cell >= ncell) return fail(ctx, DP_ERR_ARG, "side_cell out of range");
  if (tp->n_nodes <= 0 || !tp->node_energy || !tp->node_charge || !tp->node_weight)
    return fail(ctx, DP_ERR_ARG, "energy nodes required");
  if (n_rays < 0 || (n_rays > 0 && (!rays || !rho || !flux))) return fail(ctx, DP_ERR_ARG, "bad arrays");
  if (n_rays == 0) return DP_OK;
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  Inputs d;
  int rc = upload_inputs(ctx, tp, ncell, n_rays, rays, rho, cot, grad != nullptr, d);
  if (rc) return rc;
  // one-shot paths (and the FP64 Jacobian) in scratch slot 3
  const size_t cap = size_t(std::min(1001, gr->nx + gr->ny + gr->nz + 64) + 1);
  size_t bound = size_t(n_rays) * cap;  // segments cannot exceed this
  size_t need = size_t(n_rays) * cap * 12 + bound * (4 + 8 + 4 + 4 + 4 + 8) + size_t(ncell + 1) * 28 +
                size_t(n_rays + 2) * (8 + 16 + 8 + 4) + size_t(ncell / kScan + n_rays / kScan + 8) * 16 +
                64 * 256;
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, need, 3));
  A.cap = ctx->slot_bytes[3];
  if (!A.base) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  dp_paths* pa = nullptr;
  rc = build_paths(ctx, *gr, d.rays, n_rays, tp->side_cell, false, &pa, &A);
  if (rc) return rc;
  pa->rays = d.rays;
  double* djac = nullptr;
  if (row_ptr) {
    *nnz = pa->nnz;
    if (pa->nnz > nnz_cap) {
      delete pa;
      return fail(ctx, DP_ERR_ARG, "nnz_cap too small");
    }
    djac = A.take<double>(pa->nnz + 1);
    if (!djac) {
      delete pa;
      return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
    }
  }
  rc = eval_core(ctx, ph, pa, tp, d.rho, d.nE, d.nq, d.nw, d.cot, d.flux, d.grad, djac, precision);
  if (!rc) {
    cudaMemcpyAsync(flux, d.flux, 8 * n_rays, cudaMemcpyDeviceToHost, ctx->stream);
    if (grad) cudaMemcpyAsync(grad, d.grad, 8 * ncell, cudaMemcpyDeviceToHost, ctx->stream);
    if (row_ptr) {
      cudaMemcpyAsync(row_ptr, pa->row_ptr, 8 * (n_rays + 1), cudaMemcpyDeviceToHost, ctx->stream);
      if (col) cudaMemcpyAsync(col, pa->cell, 4 * pa->nnz, cudaMemcpyDeviceToHost, ctx->stream);
      if (val) cudaMemcpyAsync(val, djac, 8 * pa->nnz, cudaMemcpyDeviceToHost, ctx->stream);
    }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = fail(ctx, DP_ERR_CUDA, "download failed");
  }
  delete pa;  // arena-backed arrays: nothing to free
  return rc;
}
}  // namespace

extern "C" {

int dp_tomo_paths_create(dp_ctx* ctx, const dp_grid* gr, long n_rays, const dp_ray* rays,
                         int side_cell, dp_paths** out) {
  if (!ctx || !gr || !out || n_rays < 0 || (n_rays > 0 && !rays)) return fail(ctx, DP_ERR_ARG, "bad arguments");
  if (gr->nx <= 0 || gr->ny <= 0 || gr->nz <= 0 || !(gr->dx > 0) || !(gr->dy > 0) || !(gr->dz > 0))
    return fail(ctx, DP_ERR_ARG, "invalid grid");
  if (side_cell >= long(gr->nx) * gr->ny * gr->nz) return fail(ctx, DP_ERR_ARG, "side_cell out of range");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  dp_ray* d = nullptr;
  if (cudaMalloc(&d, sizeof(dp_ray) * (n_rays ? n_rays : 1)) != cudaSuccess)
    return fail(ctx, DP_ERR_ALLOC, "device allocation failed");
  cudaMemcpyAsync(d, rays, sizeof(dp_ray) * n_rays, cudaMemcpyHostToDevice, ctx->stream);
  int rc = build_paths(ctx, *gr, d, n_rays, side_cell, false, out);
  if (rc) {
    cudaFree(d);
    return rc;
  }
  (*out)->rays = d;  // owned by the handle
  return DP_OK;
}

int dp_tomo_eval(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa, const dp_tomo_params* tp,
                 const double* rho, const double* cot, double* flux, double* grad, double* jac) {
  if (!ctx || !ph || !pa || !tp || !rho || !flux) return fail(ctx, DP_ERR_ARG, "null argument");
  if ((cot == nullptr) != (grad == nullptr)) return fail(ctx, DP_ERR_ARG, "cot and grad go together");
  if (tp->n_nodes <= 0 || !tp->node_energy || !tp->node_charge || !tp->node_weight)
    return fail(ctx, DP_ERR_ARG, "energy nodes required");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  long ncell = long(pa->grid.nx) * pa->grid.ny * pa->grid.nz;
  // the energy nodes: uploaded once and kept on the context while calls pass
  // the same ones (three fewer round trips per call)
  const int nn = tp->n_nodes;
  bool same = ctx->nodes_dev && ctx->nodes_host.size() == size_t(3 * nn);
  for (int k = 0; same && k < nn; ++k)
    same = ctx->nodes_host[k] == tp->node_energy[k] &&
           ctx->nodes_host[nn + k] == tp->node_charge[k] &&
           ctx->nodes_host[2 * nn + k] == tp->node_weight[k];
  if (!same) {
    if (ctx->nodes_dev && ctx->nodes_host.size() != size_t(3 * nn)) {
      DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      cudaFree(ctx->nodes_dev);
      ctx->nodes_dev = nullptr;
    }
    ctx->nodes_host.clear();
    if (!ctx->nodes_dev &&
        cudaMalloc(&ctx->nodes_dev, sizeof(double) * 3 * size_t(nn)) != cudaSuccess) {
      ctx->nodes_dev = nullptr;
      return fail(ctx, DP_ERR_ALLOC, "node array allocation failed");
    }
    std::vector<double> packed(tp->node_energy, tp->node_energy + nn);
    packed.insert(packed.end(), tp->node_charge, tp->node_charge + nn);
    packed.insert(packed.end(), tp->node_weight, tp->node_weight + nn);
    // a pageable source is staged before the call returns
    DP_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->nodes_dev, packed.data(), 8 * packed.size(),
                                       cudaMemcpyHostToDevice, ctx->stream));
    ctx->nodes_host.swap(packed);
  }
  const size_t need = 8 * size_t(2 * ncell + 2 * pa->n_rays) + 8 * 256;
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, need, 2));
  A.cap = ctx->slot_bytes[2];
  double *d_rho = A.take<double>(ncell), *d_flux = A.take<double>(pa->n_rays);
  double *d_cot = cot ? A.take<double>(pa->n_rays) : nullptr;
  double *d_grad = grad ? A.take<double>(ncell) : nullptr;
  if (!d_flux || (cot && !d_cot) || (grad && !d_grad))
    return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(d_rho, rho, 8 * ncell, cudaMemcpyHostToDevice, ctx->stream));
  if (cot)
    DP_CHECK_CUDA(ctx, cudaMemcpyAsync(d_cot, cot, 8 * pa->n_rays, cudaMemcpyHostToDevice,
                                       ctx->stream));
  double* djac = nullptr;
  if (jac) {
    djac = static_cast<double*>(scratch(ctx, size_t(pa->nnz + 1) * 8, 3));
    if (!djac) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  }
  // one synchronisation at the end: the error flag comes back with the results
  const int saved = ctx->blocking;
  ctx->blocking = 0;
  const double* nd = ctx->nodes_dev;
  int rc = eval_core(ctx, ph, pa, tp, d_rho, nd, nd + nn, nd + 2 * nn, d_cot, d_flux, d_grad,
                     djac, tp->precision);
  ctx->blocking = saved;
  if (rc) return rc;
  int flag = 0;
  cudaMemcpyAsync(flux, d_flux, 8 * pa->n_rays, cudaMemcpyDeviceToHost, ctx->stream);
  if (grad) cudaMemcpyAsync(grad, d_grad, 8 * ncell, cudaMemcpyDeviceToHost, ctx->stream);
  if (jac) cudaMemcpyAsync(jac, djac, 8 * pa->nnz, cudaMemcpyDeviceToHost, ctx->stream);
  if (saved) cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return fail(ctx, DP_ERR_STATE,
                flag == 2 ? "ray segment buffer overflow" : "table-staging wait exceeded its limit");
  }
  return DP_OK;
}

int dp_tomo_paths_create_dev(dp_ctx* ctx, const dp_grid* gr, long n_rays, const dp_ray* rays,
                             int side_cell, dp_paths** out) {
  if (!ctx || !gr || !out || n_rays < 0 || (n_rays > 0 && !rays)) return fail(ctx, DP_ERR_ARG, "bad arguments");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  return build_paths(ctx, *gr, rays, n_rays, side_cell, true, out);
}

int dp_tomo_paths_free(dp_paths* p) {
  if (!p) return DP_ERR_ARG;
  cudaSetDevice(p->device);  // the context may already be destroyed
  free_paths_arrays(p);
  cudaGetLastError();  // a failed release must not surface at a later launch
  delete p;
  return DP_OK;
}

int dp_tomo_paths_info(const dp_paths* p, long* n_rays, int64_t* nnz, int* max_segments) {
  if (!p) return DP_ERR_ARG;
  if (n_rays) *n_rays = p->n_rays;
  if (nnz) *nnz = p->nnz;
  if (max_segments) *max_segments = p->max_seg;
  return DP_OK;
}

int dp_tomo_paths_csr(const dp_paths* p, int64_t* row_ptr, int32_t* col, double* len) {
  if (!p) return DP_ERR_ARG;
  cudaSetDevice(p->device);
  if (row_ptr) cudaMemcpy(row_ptr, p->row_ptr, 8 * (p->n_rays + 1), cudaMemcpyDeviceToHost);
  if (col) cudaMemcpy(col, p->cell, 4 * p->nnz, cudaMemcpyDeviceToHost);
  if (len) cudaMemcpy(len, p->len, 8 * p->nnz, cudaMemcpyDeviceToHost);
  return DP_OK;
}

int dp_tomo_eval_dev(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa, const dp_tomo_params* tp,
                     const double* rho, const double* cot, double* flux, double* grad, double* jac,
                     int precision) {
  if (!ctx || !pa || !tp || !rho || !flux) return fail(ctx, DP_ERR_ARG, "null argument");
  if ((cot == nullptr) != (grad == nullptr)) return fail(ctx, DP_ERR_ARG, "cot and grad go together");
  if (precision != 0 && precision != 1) return fail(ctx, DP_ERR_ARG, "precision must be 0 or 1");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  return eval_core(ctx, ph, pa, tp, rho, tp->node_energy, tp->node_charge, tp->node_weight, cot, flux,
                   grad, jac, precision);
}

int dp_tomo_forward(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                    const double* rho, long n_rays, const dp_ray* rays, double* flux) {
  return host_eval(ctx, ph, gr, tp, rho, n_rays, rays, nullptr, flux, nullptr, nullptr, nullptr,
                   nullptr, 0, nullptr, tp ? tp->precision : 0);
}

int dp_tomo_jacobian(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                     const double* rho, long n_rays, const dp_ray* rays, double* flux, int64_t* row_ptr,
                     int32_t* col, double* val, int64_t nnz_cap, int64_t* nnz) {
  if (!row_ptr || !nnz) return fail(ctx, DP_ERR_ARG, "row_ptr and nnz required");
  return host_eval(ctx, ph, gr, tp, rho, n_rays, rays, nullptr, flux, nullptr, row_ptr, col, val,
                   nnz_cap, nnz, tp ? tp->precision : 0);
}

int dp_tomo_vjp(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                const double* rho, long n_rays, const dp_ray* rays, const double* cot, double* flux,
                double* grad) {
  if (!cot || !grad) return fail(ctx, DP_ERR_ARG, "cot and grad required");
  return host_eval(ctx, ph, gr, tp, rho, n_rays, rays, cot, flux, grad, nullptr, nullptr, nullptr, 0,
                   nullptr, tp ? tp->precision : 0);
}

int dp_tomo_forward_plain_dev(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr,
                              const dp_tomo_params* tp, const double* rho, long n_rays,
                              const dp_ray* rays, double* flux) {
  if (!ctx || !ph || !gr || !tp || n_rays < 0) return fail(ctx, DP_ERR_ARG, "null argument");
  if (tp->n_nodes <= 0 || tp->n_nodes > 1024) return fail(ctx, DP_ERR_ARG, "1..1024 nodes");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  double* part = static_cast<double*>(scratch(ctx, size_t(n_rays) * tp->n_nodes * 8, 0));
  if (!part) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  EvalP P{};
  P.tab = ph->view;
  P.rock = tp->rock_material;
  P.air = tp->air_material;
  P.n_nodes = tp->n_nodes;
  P.H = tp->primary_altitude > 0 ? tp->primary_altitude : 3e4;
  P.mass = ph->settings.mass;
  P.ctau = ph->settings.ctau;
  GridDev g = grid_dev(*gr);
  P.zmax = g.zmax;
  P.air_dexp = std::exp(-P.zmax / 12e3) - std::exp(-P.H / 12e3);
  P.side_density = tp->side_density;
  P.rho = rho;
  P.rays = rays;
  P.nE = tp->node_energy;
  P.nq = tp->node_charge;
  P.nw = tp->node_weight;
  for (long r = 0; r < n_rays; ++r)
    plain_ray_kernel<<<1, tp->n_nodes, 0, ctx->stream>>>(P, g, tp->side_cell, r, part);
  plain_sum_kernel<<<int((n_rays + 127) / 128), 128, 0, ctx->stream>>>(part, n_rays, tp->n_nodes, flux);
  ctx->launches += n_rays + 1;
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  return check(ctx);
}

// Deprecated single-shot device form kept for callers of the first ABI version.
int dp_tomo_vjp_dev(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                    const double* rho, long n_rays, const dp_ray* rays, const double* cot,
                    double* flux, double* grad) {
  dp_paths* pa = nullptr;
  int rc = dp_tomo_paths_create_dev(ctx, gr, n_rays, rays, tp ? tp->side_cell : -1, &pa);
  if (rc) return rc;
  rc = dp_tomo_eval_dev(ctx, ph, pa, tp, rho, cot, flux, grad, nullptr, tp->precision);
  dp_tomo_paths_free(pa);
  return rc;
}

}  // extern "C"

// ============================================================ allocation-free evaluation
// Some callers may not allocate device memory during a call: a long-running
// service that holds a fixed device-memory budget, or a plugin whose host
// process owns all device memory through its own pool allocator (a stray
// cudaMalloc would fragment or exceed it).  dp_tomo_eval_noalloc_dev serves
// them: it evaluates the mixed-precision flux and J^T r on resident paths and
// keeps its only scratch -- the per-segment Jacobian values -- in the
// file-scope array below instead of the context's grow-on-demand scratch.
// The array is a fixed part of the library: every GPU that loads libdpgpu
// holds it (8 MiB) until the process exits.
namespace dp {
constexpr long kNoAllocMaxSegments = 1L << 21;  // 2,097,152 segments, FP32 values
static __device__ __align__(256) float g_noalloc_jacobian[kNoAllocMaxSegments];

// Device address of g_noalloc_jacobian, looked up once per device with that
// device current (the host-side symbol is only a stand-in, never a device
// address).  The address belongs to the device's primary context, the one
// the CUDA runtime uses: it stays valid until the process exits unless the
// caller resets the device (cudaDeviceReset), after which this entry point
// must not be called again in the process.
static float* noalloc_scratch(int device, cudaError_t* err) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static float* addr[kMaxDevices] = {};
  *err = cudaSuccess;
  if (device < 0 || device >= kMaxDevices) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    float* p = nullptr;
    *err = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_jacobian);
    if (*err != cudaSuccess) return nullptr;
    addr[device] = p;
  }
  return addr[device];
}
}  // namespace dp

extern "C" int dp_tomo_eval_noalloc_dev(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa,
                                        const dp_tomo_params* tp, const double* rho,
                                        const double* cot, double* flux, double* grad) {
  if (!ctx || !ph || !pa || !tp || !rho || !flux) return fail(ctx, DP_ERR_ARG, "null argument");
  if ((cot == nullptr) != (grad == nullptr)) return fail(ctx, DP_ERR_ARG, "cot and grad go together");
  if (pa->nnz > kNoAllocMaxSegments)
    return fail(ctx, DP_ERR_ARG,
                "dp_tomo_eval_noalloc_dev: the paths hold " + std::to_string(pa->nnz) +
                    " segments, more than its fixed scratch of " + std::to_string(kNoAllocMaxSegments) +
                    "; use dp_tomo_eval_dev");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaError_t e;
  float* jac = noalloc_scratch(ctx->device, &e);
  if (!jac) return cuda_fail(ctx, e, "cudaGetSymbolAddress(g_noalloc_jacobian)");
  EvalP P;
  int rc = make_eval(ctx, ph, pa, tp, P);
  if (rc) return rc;
  if (pa->n_rays == 0) return DP_OK;
  P.rho = rho;
  P.nE = tp->node_energy;
  P.nq = tp->node_charge;
  P.nw = tp->node_weight;
  P.flux = flux;
  P.jval32 = jac;  // every segment's value is written before the gather reads it
  const size_t smem = size_t(2 * kNC32) * P.ld32 * 4 + size_t(kWarps) * P.seg_cap * 3 * 4 +
                      size_t(P.n_nodes) * sizeof(NodeInit);
  if (smem > 220 * 1024) return fail(ctx, DP_ERR_ARG, "ray too long for the mixed kernel");
  const long blocks = std::min<long>((pa->n_rays + kWarps - 1) / kWarps, 152L * 16);
  const bool adj = cot != nullptr;
  if (adj) {
    DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(eval32_kernel<true>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    eval32_kernel<true><<<int(blocks), kWarps * 32, smem, ctx->stream>>>(P);
  } else {
    DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(eval32_kernel<false>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    eval32_kernel<false><<<int(blocks), kWarps * 32, smem, ctx->stream>>>(P);
  }
  ++ctx->launches;
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  if (adj) {
    const long ncell = long(pa->grid.nx) * pa->grid.ny * pa->grid.nz;
    gather_small_kernel<float><<<int((ncell + 255) / 256), 256, 0, ctx->stream>>>(
        pa->cptr, pa->perm, jac, pa->prow, cot, ncell, grad);
    ++ctx->launches;
    if (pa->n_big > 0) {
      gather_big_kernel<float><<<pa->n_big, kBigThreads, 0, ctx->stream>>>(
          pa->cptr, pa->perm, jac, pa->prow, cot, pa->big, pa->n_big, grad);
      ++ctx->launches;
    }
    DP_CHECK_CUDA(ctx, cudaGetLastError());
  }
  return check(ctx);
}

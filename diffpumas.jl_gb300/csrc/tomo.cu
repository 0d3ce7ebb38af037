// tomo.cu -- voxel-density tomography forward model and its density adjoint.
//
// Forward (examples/diff_flux_cube.jl:304-470): the ray is marched through
// the grid exactly as trace_cube_path does it (position-based boundary march,
// candidates x, y, z with strict improvement, 1e-10 tolerance, 1 cm nudge),
// so the segment list is identical to the reference's; the march uses
// correctly rounded FP64 operations without contraction.  Per energy node,
// each segment inverts the CSDA range (X = R(E), E' = R^-1(X + rho L)),
// multiplies the weight by S(E')/S(E) and the decay factor, the side-exit
// remainder and the closed-form air column follow, then the GCCLY flux.
//
// Adjoint: one warp per ray, one lane per energy node.  A reverse sweep over
// the segment list recomputes the per-segment energies and carries
// lambda_k = d log(flux)/d E_k; d flux/d rho_k = flux lambda_k dE_k/dY_k L_k.
// Lanes are reduced per segment with a fixed shuffle tree, giving one Jacobian
// entry per traversed segment (CSR).  J^T r is formed by a deterministic
// segmented reduction: entries are bucketed by cell (integer counts), each
// bucket is ordered by entry index, then summed in that order -- no
// floating-point atomics, bitwise reproducible.
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace dp {

struct GridDev {
  int nx, ny, nz;
  double x0, y0, z0, dx, dy, dz, xmax, ymax, zmax;
};

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

// examples/diff_flux_cube.jl:304-366 (trace_cube_path).  Calls emit(cell, L)
// per segment; returns the number of segments, or -1 past `cap`; *z_exit gets
// the last segment end height.
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

struct TomoDev {
  TabView tab;
  GridDev g;
  int rock, air, side_cell, n_nodes, seg_cap;
  double side_density, H, mass, ctau, air_dexp;  // exp(-zmax/h) - exp(-H/h)
  const double *nE, *nq, *nw;  // device node arrays
  const double* rho;
  const dp_ray* rays;
  long n_rays;
  double* flux;
  const int64_t* row_ptr;  // MODE 1
  int32_t* col;
  double* val;
  int32_t* row_of;
  int* err_flag;
};

// Per-segment decay exponent derivative: d log D / d Eavg for
// D = exp(-L / (beta gamma ctau)), beta = sqrt(max(1 - 1/gamma^2, 1e-12)).
__device__ __forceinline__ double decay_log(double L, double Eavg, double mass, double ctau,
                                            double* dlog) {
  double g = 1.0 + Eavg / mass, b2 = 1.0 - 1.0 / (g * g);
  bool clamp = !(b2 > 1e-12);
  double b = sqrt(clamp ? 1e-12 : b2), bg = b * g;
  if (dlog) *dlog = L / (ctau * bg * bg) * (clamp ? b : 1.0 / b) / mass;
  return -L / (bg * ctau);
}

// log-derivative helpers on the staged tables
__device__ __forceinline__ double dlogS(const TabView& t, const double* E, const double* lE,
                                        const double* S, double e, double* Sval) {
  Dd s = interp_logE(t, E, lE, S, dd(e, 1.0 / e), dd(log(e), 1.0 / e), nullptr);
  *Sval = s.v;
  return s.d / s.v;
}
__device__ __forceinline__ double range_slope(const TabView& t, const double* E, const double* lE,
                                              const double* R, double e) {
  // dR/dE (zero outside the table, rrule convention)
  return interp_logE(t, E, lE, R, dd(e, 1.0), dd(log(e), 1.0 / e), nullptr).d;
}
__device__ __forceinline__ double inv_slope(const double* R, const double* E, const double* lE,
                                            int n, double Y) {
  return inverse_range(R, E, lE, n, dd(Y, 1.0), nullptr).d;
}

enum { T_E = 0, T_LOGE, T_RS, T_RR, T_AS, T_AR, T_NCOL };

template <int MODE>
__global__ void __launch_bounds__(128) tomo_kernel(TomoDev P) {
  extern __shared__ __align__(16) double smem[];
  __shared__ uint64_t mbar;
  const int ld = P.tab.ld, n = P.tab.n;
  const double* src[T_NCOL] = {P.tab.col(0, DP_COL_E),          P.tab.col(0, DP_COL_LOGE),
                               P.tab.col(P.rock, DP_COL_CSDA_S), P.tab.col(P.rock, DP_COL_CSDA_R),
                               P.tab.col(P.air, DP_COL_CSDA_S),  P.tab.col(P.air, DP_COL_CSDA_R)};
  if (!stage_columns(smem, src, T_NCOL, uint32_t(ld * sizeof(double)), &mbar)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    return;
  }
  const double *tE = smem + T_E * ld, *tlE = smem + T_LOGE * ld;
  const double *rS = smem + T_RS * ld, *rR = smem + T_RR * ld;
  const double *aS = smem + T_AS * ld, *aR = smem + T_AR * ld;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cap = P.seg_cap;
  // per-warp segment buffers after the tables: length, density, Jacobian
  // accumulator (doubles), then cell ids (ints)
  double* wbase = smem + T_NCOL * ld + size_t(warp) * cap * 3;
  double* sL = wbase;
  double* sD = wbase + cap;
  double* sJ = wbase + 2 * cap;
  int* cells = reinterpret_cast<int*>(smem + T_NCOL * ld + size_t(4) * cap * 3) + size_t(warp) * cap;
  const double Emax = tE[n - 1];
  for (long r = blockIdx.x * 4L + warp; r < P.n_rays; r += gridDim.x * 4L) {
    dp_ray ray = P.rays[r];
    double z_exit;
    int ns = trace(P.g, ray, cap - 1, &z_exit, [&](int s, int cell, double L) {
      if (lane == 0) {
        cells[s] = cell;
        sL[s] = L;
        sD[s] = P.rho[cell];
      }
    });
    if (ns < 0) {
      if (lane == 0) atomicExch(P.err_flag, 2);
      continue;
    }
    // side-exit remainder as one more rock segment (diff_flux_cube.jl:417-444)
    const double cs_safe = fmax(fabs(ray.cos_theta), 0.01);
    bool side = z_exit < P.g.zmax - kEps64;
    if (side && lane == 0) {
      cells[ns] = P.side_cell;
      sL[ns] = (P.g.zmax - z_exit) / cs_safe;
      sD[ns] = P.side_cell >= 0 ? P.rho[P.side_cell] : P.side_density;
    }
    const int nseg = ns + (side ? 1 : 0);
    if (MODE == 1)
      for (int s = lane; s < nseg; s += 32) sJ[s] = 0.0;
    __syncwarp();
    const double Lair = (P.H - P.g.zmax) / cs_safe;
    const double Gair = fmax((1.205 * 12e3 / cs_safe) * P.air_dexp, 0.0);
    const double cs = cos_theta_star(ray.cos_theta), cs129 = pow(cs, 1.29);
    double fsum = 0.0;
    for (int base = 0; base < P.n_nodes; base += 32) {
      const int nd = base + lane;
      const bool active = nd < P.n_nodes;
      double E = active ? P.nE[nd] : 1.0;
      double w = 1.0;
      bool ok = active;
      int kc = -1;
      double Eprev_c = 0.0;
      int hint = 0;
      for (int s = 0; s < nseg && ok; ++s) {
        double X = interp_logE(P.tab, tE, tlE, rR, dd(E), dd(log(E)), nullptr).v;
        double Ek = inverse_range(rR, tE, tlE, n, dd(X + sL[s] * sD[s]), &hint).v;
        if (!(Ek < 1e12) || !isfinite(Ek)) {
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
        if (Ef < 1e12 && isfinite(Ef)) {
          double Sa0 = interp_logE(P.tab, tE, tlE, aS, dd(E), dd(log(E)), nullptr).v;
          double Sa1 = interp_logE(P.tab, tE, tlE, aS, dd(Ef), dd(log(Ef)), nullptr).v;
          w = w * (Sa1 / Sa0);
          w = w * exp(decay_log(Lair, (E + Ef) / 2.0, P.mass, P.ctau, nullptr));
          f = w * gccly_flux(cs, cs129, Ef, active ? P.nq[nd] : 0.0, nullptr);
        } else {
          ok = false;
        }
      }
      const double coef = active && ok ? 2.0 * P.nw[nd] / P.n_nodes : 0.0;
      fsum += coef * f;
      if (MODE == 1) {
        // ---- reverse sweep
        double lam = 0.0;
        if (coef != 0.0 && f != 0.0) {
          double Sv;
          double aA;
          decay_log(Lair, (EN + Ef) / 2.0, P.mass, P.ctau, &aA);
          double dlogF;
          gccly_flux(cs, cs129, Ef, P.nq[nd], &dlogF);
          double dEf = inv_slope(aR, tE, tlE, n,
                                 interp_logE(P.tab, tE, tlE, aR, dd(EN), dd(log(EN)), nullptr).v +
                                     Gair) *
                       range_slope(P.tab, tE, tlE, aR, EN);
          lam = dlogS(P.tab, tE, tlE, rS, EN, &Sv) - dlogS(P.tab, tE, tlE, aS, EN, &Sv) + 0.5 * aA +
                dEf * (dlogS(P.tab, tE, tlE, aS, Ef, &Sv) + 0.5 * aA + dlogF);
        }
        double Ek = EN;
        int hint_r = n - 2;
        for (int s = nseg - 1; s >= 0; --s) {
          double v = 0.0, Ekm1 = 0.0, a = 0.0;
          if (coef != 0.0 && f != 0.0) {
            const double L = sL[s], Y = interp_logE(P.tab, tE, tlE, rR, dd(Ek), dd(log(Ek)), nullptr).v;
            if (kc >= 0 && s > kc) Ekm1 = Emax;
            else if (s == kc) Ekm1 = Eprev_c;
            else {
              // walk down from the previous interval (energies decrease)
              Ekm1 = inverse_range(rR, tE, tlE, n, dd(Y - L * sD[s]), nullptr).v;
            }
            (void)hint_r;
            double Ycur = interp_logE(P.tab, tE, tlE, rR, dd(Ekm1), dd(log(Ekm1)), nullptr).v + L * sD[s];
            double Kp = (Ek >= Emax) ? 0.0 : inv_slope(rR, tE, tlE, n, Ycur);
            decay_log(L, (Ekm1 + Ek) / 2.0, P.mass, P.ctau, &a);
            lam += 0.5 * a;  // decay of this segment through E_k
            v = coef * f * lam * Kp * L;
            // propagate to E_{k-1}
            double Rp = range_slope(P.tab, tE, tlE, rR, Ekm1);
            lam = lam * Kp * Rp + 0.5 * a;
          }
          // deterministic lane reduction
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if (lane == 0) sJ[s] += v;
          Ek = Ekm1;
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
    if (lane == 0) P.flux[r] = fsum;
    if (MODE == 1) {
      __syncwarp();
      const int64_t off = P.row_ptr[r];
      const int nent = int(P.row_ptr[r + 1] - off);
      for (int s = lane; s < nseg && s < nent; s += 32) {
        P.col[off + s] = cells[s];
        P.val[off + s] = sJ[s];
        if (P.row_of) P.row_of[off + s] = int32_t(r);
      }
    }
    __syncwarp();
  }
}

// Segment count per ray (+1 for a side exit), one thread per ray.
__global__ void tomo_count_kernel(GridDev g, const dp_ray* rays, long n_rays, int cap,
                                  int64_t* counts, int* err_flag) {
  long r = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (r >= n_rays) return;
  double z_exit;
  dp_ray ray = rays[r];
  int ns = trace(g, ray, cap - 1, &z_exit, [](int, int, double) {});
  if (ns < 0) {
    atomicExch(err_flag, 2);
    ns = 0;
  }
  counts[r] = ns + (z_exit < g.zmax - kEps64 ? 1 : 0);
}

// Exclusive scan of int64 (two levels; the second level walks any number of
// block totals serially in one block).
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

// J^T r: bucket entries by cell.
__global__ void hist_kernel(const int32_t* col, long nnz, int32_t* count) {
  long e = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (e < nnz && col[e] >= 0) atomicAdd(&count[col[e]], 1);
}
__global__ void i32_to_i64(const int32_t* a, int64_t* b, long n) {
  long i = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (i < n) b[i] = a[i];
}
__global__ void place_kernel(const int32_t* col, long nnz, const int64_t* cptr, int32_t* cursor,
                             int32_t* perm) {
  long e = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (e >= nnz || col[e] < 0) return;
  int c = col[e];
  perm[cptr[c] + atomicAdd(&cursor[c], 1)] = int32_t(e);
}
// One thread per cell: order its bucket by entry index, then sum in order.
__global__ void gather_kernel(const int64_t* cptr, int32_t* perm, const double* val,
                              const int32_t* row_of, const double* cot, long ncell, double* grad) {
  long c = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (c >= ncell) return;
  int64_t b = cptr[c], e = cptr[c + 1];
  for (int64_t i = b + 1; i < e; ++i) {
    int32_t x = perm[i];
    int64_t j = i - 1;
    while (j >= b && perm[j] > x) {
      perm[j + 1] = perm[j];
      --j;
    }
    perm[j + 1] = x;
  }
  double s = 0.0;
  for (int64_t i = b; i < e; ++i) s += val[perm[i]] * cot[row_of[perm[i]]];
  grad[c] = s;
}

// ---------------------------------------------------------------- plain form
// Plain FP64 form: one launch per ray, one thread per node, global tables,
// bisection lookups, no staging.
__global__ void plain_ray_kernel(TomoDev P, long r) {
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
  trace(P.g, ray, 1 << 30, &z_exit, [&](int, int cell, double L) { seg(P.rho[cell], L); });
  double cs_safe = fmax(fabs(ray.cos_theta), 0.01);
  if (z_exit < P.g.zmax - kEps64)
    seg(P.side_cell >= 0 ? P.rho[P.side_cell] : P.side_density, (P.g.zmax - z_exit) / cs_safe);
  double f = 0.0;
  if (ok) {
    double Xa = interp_logE(tb, E_, lE, aR, dd(E), dd(log(E)), nullptr).v;
    double Gair = fmax((1.205 * 12e3 / cs_safe) * P.air_dexp, 0.0);
    double Ef = inverse_range(aR, E_, lE, t.n, dd(Xa + Gair), nullptr).v;
    w *= interp_logE(tb, E_, lE, aS, dd(Ef), dd(log(Ef)), nullptr).v /
         interp_logE(tb, E_, lE, aS, dd(E), dd(log(E)), nullptr).v;
    w *= exp(decay_log((P.H - P.g.zmax) / cs_safe, (E + Ef) / 2.0, P.mass, P.ctau, nullptr));
    double cs = cos_theta_star(ray.cos_theta);
    f = w * gccly_flux(cs, pow(cs, 1.29), Ef, P.nq[nd], nullptr);
  }
  // per-node result; the host-side sum is part of the plain form
  P.val[r * P.n_nodes + nd] = 2.0 * P.nw[nd] * f / P.n_nodes;
}
__global__ void plain_sum_kernel(const double* v, long n_rays, int n_nodes, double* flux) {
  long r = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (r >= n_rays) return;
  double s = 0.0;
  for (int k = 0; k < n_nodes; ++k) s += v[r * n_nodes + k];
  flux[r] = s;
}

// ---------------------------------------------------------------- host side
struct Scratch {
  char* p;
  size_t off = 0;
  template <class T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* r = reinterpret_cast<T*>(p + off);
    off += n * sizeof(T);
    return r;
  }
};

static int make_params(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                       TomoDev& P) {
  if (!ctx || !ph || !gr || !tp) return fail(ctx, DP_ERR_ARG, "null argument");
  if (gr->nx <= 0 || gr->ny <= 0 || gr->nz <= 0 || !(gr->dx > 0) || !(gr->dy > 0) || !(gr->dz > 0))
    return fail(ctx, DP_ERR_ARG, "invalid grid");
  if (tp->n_nodes <= 0 || !tp->node_energy || !tp->node_charge || !tp->node_weight)
    return fail(ctx, DP_ERR_ARG, "energy nodes required");
  if (tp->rock_material < 0 || tp->rock_material >= ph->n_mat || tp->air_material < 0 ||
      tp->air_material >= ph->n_mat)
    return fail(ctx, DP_ERR_ARG, "material index out of range");
  long ncell = long(gr->nx) * gr->ny * gr->nz;
  if (tp->side_cell >= ncell) return fail(ctx, DP_ERR_ARG, "side_cell out of range");
  P = TomoDev{};
  P.tab = ph->view;
  P.g = GridDev{gr->nx, gr->ny, gr->nz, gr->x0, gr->y0, gr->z0, gr->dx, gr->dy, gr->dz,
                gr->x0 + gr->nx * gr->dx, gr->y0 + gr->ny * gr->dy, gr->z0 + gr->nz * gr->dz};
  P.rock = tp->rock_material;
  P.air = tp->air_material;
  P.side_cell = tp->side_cell;
  P.side_density = tp->side_density;
  P.H = tp->primary_altitude > 0 ? tp->primary_altitude : 3e4;
  P.mass = ph->settings.mass;
  P.ctau = ph->settings.ctau;
  P.n_nodes = tp->n_nodes;
  // the reference march stops after 1000 steps; one segment per crossed plane
  P.seg_cap = std::min(1001, gr->nx + gr->ny + gr->nz + 64) + 1;
  P.air_dexp = std::exp(-P.g.zmax / 12e3) - std::exp(-P.H / 12e3);
  P.err_flag = ctx->d_flag;
  return DP_OK;
}

static int check(dp_ctx* ctx) {
  int flag = 0;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return fail(ctx, DP_ERR_STATE, flag == 2 ? "ray segment buffer overflow" : "table-staging wait exceeded its limit");
  }
  return DP_OK;
}

static size_t tomo_smem(const TomoDev& P) {
  return size_t(T_NCOL) * P.tab.ld * sizeof(double) + size_t(4) * P.seg_cap * (3 * sizeof(double) + sizeof(int));
}

// Device-pointer core.  cot == nullptr: forward only.  Jacobian outputs when
// row_ptr/col/val are given (device).  grad: J^T cot.
static int tomo_core(dp_ctx* ctx, TomoDev& P, long n_rays, const dp_ray* rays, const double* rho,
                     const double* nE, const double* nq, const double* nw, double* flux,
                     const double* cot, double* grad, int64_t* row_ptr_out, int32_t* col_out,
                     double* val_out, int64_t nnz_cap, int64_t* nnz_out) {
  P.rays = rays;
  P.n_rays = n_rays;
  P.rho = rho;
  P.nE = nE;
  P.nq = nq;
  P.nw = nw;
  P.flux = flux;
  size_t smem = tomo_smem(P);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(tomo_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(tomo_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  long blocks = (n_rays + 3) / 4;
  if (blocks > 152L * 8) blocks = 152L * 8;
  const bool need_j = cot || row_ptr_out;
  if (!need_j) {
    timed_begin(ctx);
    tomo_kernel<0><<<int(blocks), 128, smem, ctx->stream>>>(P);
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "tomo_forward");
    return check(ctx);
  }
  long ncell = long(P.g.nx) * P.g.ny * P.g.nz;
  long nbr = (n_rays + 1 + kScan - 1) / kScan;
  // slot 0: per-ray arrays; slot 1: per-entry and per-cell arrays
  size_t est = size_t(n_rays + 2) * 8 * 2 + size_t(nbr + 2) * 8 + 4096;
  Scratch s0{static_cast<char*>(scratch(ctx, est, 0))};
  if (!s0.p) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  int64_t* counts = s0.take<int64_t>(n_rays + 1);
  int64_t* rptr = row_ptr_out ? row_ptr_out : s0.take<int64_t>(n_rays + 1);
  int64_t* totals = s0.take<int64_t>(nbr + 2);
  int64_t* grand = totals + nbr + 1;
  tomo_count_kernel<<<int((n_rays + 127) / 128), 128, 0, ctx->stream>>>(P.g, rays, n_rays, P.seg_cap,
                                                                          counts, ctx->d_flag);
  scan_blocks<<<int(nbr), kScan, 0, ctx->stream>>>(counts, rptr, n_rays, totals);
  scan_totals<<<1, kScan, 0, ctx->stream>>>(totals, nbr, grand);
  scan_add<<<int(nbr), kScan, 0, ctx->stream>>>(rptr, n_rays, totals, grand);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  ctx->launches += 4;
  int64_t nnz = 0;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(&nnz, rptr + n_rays, 8, cudaMemcpyDeviceToHost, ctx->stream));
  int rc = check(ctx);
  if (rc) return rc;
  if (nnz_out) *nnz_out = nnz;
  if (row_ptr_out && nnz > nnz_cap) return fail(ctx, DP_ERR_ARG, "nnz_cap too small");
  long nbc = (ncell + 1 + kScan - 1) / kScan;
  size_t need = size_t(nnz + 1) * (4 + 8 + 4 + 4) + size_t(ncell + 1) * (8 + 8 + 4 + 4) +
                size_t(nbc + 2) * 8 + 16 * 256;
  Scratch s1{static_cast<char*>(scratch(ctx, need, 1))};
  if (!s1.p) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  int32_t* col = col_out ? col_out : s1.take<int32_t>(nnz + 1);
  double* val = val_out ? val_out : s1.take<double>(nnz + 1);
  int32_t* row_of = cot ? s1.take<int32_t>(nnz + 1) : nullptr;
  Scratch& s0c = s1;
  P.row_ptr = rptr;
  P.col = col;
  P.val = val;
  P.row_of = row_of;
  timed_begin(ctx);
  tomo_kernel<1><<<int(blocks), 128, smem, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "tomo_adjoint");
  if (cot && grad) {
    int32_t* ccount = s0c.take<int32_t>(ncell + 1);
    int32_t* cursor = s0c.take<int32_t>(ncell + 1);
    int64_t* ccount64 = s0c.take<int64_t>(ncell + 1);
    int64_t* cptr = s0c.take<int64_t>(ncell + 1);
    int64_t* ctot = s0c.take<int64_t>(nbc + 2);
    int32_t* perm = s0c.take<int32_t>(nnz + 1);
    DP_CHECK_CUDA(ctx, cudaMemsetAsync(ccount, 0, size_t(ncell + 1) * 4, ctx->stream));
    DP_CHECK_CUDA(ctx, cudaMemsetAsync(cursor, 0, size_t(ncell + 1) * 4, ctx->stream));
    int tb = 256;
    timed_begin(ctx);
    ctx->launches += nnz > 0 ? 6 : 4;
    if (nnz > 0) hist_kernel<<<int((nnz + tb - 1) / tb), tb, 0, ctx->stream>>>(col, nnz, ccount);
    i32_to_i64<<<int((ncell + tb - 1) / tb), tb, 0, ctx->stream>>>(ccount, ccount64, ncell);
    scan_blocks<<<int(nbc), kScan, 0, ctx->stream>>>(ccount64, cptr, ncell, ctot);
    scan_totals<<<1, kScan, 0, ctx->stream>>>(ctot, nbc, ctot + nbc + 1);
    scan_add<<<int(nbc), kScan, 0, ctx->stream>>>(cptr, ncell, ctot, ctot + nbc + 1);
    if (nnz > 0) place_kernel<<<int((nnz + tb - 1) / tb), tb, 0, ctx->stream>>>(col, nnz, cptr, cursor, perm);
    gather_kernel<<<int((ncell + tb - 1) / tb), tb, 0, ctx->stream>>>(cptr, perm, val, row_of, cot, ncell, grad);
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "tomo_transpose");
  }
  return check(ctx);
}

struct HostTomo {
  dp_ray* rays;
  double *rho, *nE, *nq, *nw, *flux, *cot, *grad;
};

}  // namespace dp

using namespace dp;

static int upload_common(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                         const double* rho, long n_rays, const dp_ray* rays, TomoDev& P,
                         std::vector<void*>& allocs, HostTomo& d) {
  int rc = make_params(ctx, ph, gr, tp, P);
  if (rc) return rc;
  if (n_rays < 0 || (n_rays > 0 && (!rays || !rho))) return fail(ctx, DP_ERR_ARG, "bad ray/density arrays");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  long ncell = long(gr->nx) * gr->ny * gr->nz;
  auto al = [&](size_t b) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, b ? b : 8) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return p;
  };
  d.rays = (dp_ray*)al(sizeof(dp_ray) * n_rays);
  d.rho = (double*)al(8 * ncell);
  d.nE = (double*)al(8 * tp->n_nodes);
  d.nq = (double*)al(8 * tp->n_nodes);
  d.nw = (double*)al(8 * tp->n_nodes);
  d.flux = (double*)al(8 * n_rays);
  for (void* p : allocs)
    if (!p) return fail(ctx, DP_ERR_ALLOC, "device allocation failed");
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(d.rays, rays, sizeof(dp_ray) * n_rays, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(d.rho, rho, 8 * ncell, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(d.nE, tp->node_energy, 8 * tp->n_nodes, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(d.nq, tp->node_charge, 8 * tp->n_nodes, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(d.nw, tp->node_weight, 8 * tp->n_nodes, cudaMemcpyHostToDevice, ctx->stream));
  return DP_OK;
}

static void free_all(std::vector<void*>& a) {
  for (void* p : a) cudaFree(p);
  a.clear();
}

// Air grammage depends only on the grid top and the ray's cos theta; it is
// evaluated per ray inside the kernel from this closed form.  The kernel gets
// the value for cos_theta of each ray through this helper applied on device.
extern "C" {

int dp_tomo_vjp_dev(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                    const double* rho, long n_rays, const dp_ray* rays, const double* cot,
                    double* flux, double* grad) {
  TomoDev P;
  int rc = make_params(ctx, ph, gr, tp, P);
  if (rc) return rc;
  if (n_rays <= 0) return n_rays == 0 ? DP_OK : fail(ctx, DP_ERR_ARG, "negative n_rays");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  // Node arrays given as device pointers in tp for this entry point.
  return tomo_core(ctx, P, n_rays, rays, rho, tp->node_energy, tp->node_charge, tp->node_weight, flux,
                   cot, grad, nullptr, nullptr, nullptr, 0, nullptr);
}

int dp_tomo_forward(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                    const double* rho, long n_rays, const dp_ray* rays, double* flux) {
  if (!flux && n_rays > 0) return fail(ctx, DP_ERR_ARG, "flux output required");
  TomoDev P;
  std::vector<void*> al;
  HostTomo d{};
  int rc = upload_common(ctx, ph, gr, tp, rho, n_rays, rays, P, al, d);
  if (rc || n_rays == 0) {
    free_all(al);
    return rc;
  }
  rc = tomo_core(ctx, P, n_rays, d.rays, d.rho, d.nE, d.nq, d.nw, d.flux, nullptr, nullptr, nullptr,
                 nullptr, nullptr, 0, nullptr);
  if (!rc && cudaMemcpy(flux, d.flux, 8 * n_rays, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = fail(ctx, DP_ERR_CUDA, "flux download failed");
  free_all(al);
  return rc;
}

int dp_tomo_jacobian(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                     const double* rho, long n_rays, const dp_ray* rays, double* flux, int64_t* row_ptr,
                     int32_t* col, double* val, int64_t nnz_cap, int64_t* nnz) {
  if (!flux || !row_ptr || !nnz || n_rays <= 0) return fail(ctx, DP_ERR_ARG, "bad output arrays");
  TomoDev P;
  std::vector<void*> al;
  HostTomo d{};
  int rc = upload_common(ctx, ph, gr, tp, rho, n_rays, rays, P, al, d);
  if (rc) {
    free_all(al);
    return rc;
  }
  int64_t* drp = nullptr;
  int32_t* dcol = nullptr;
  double* dval = nullptr;
  size_t cap = size_t(nnz_cap > 0 ? nnz_cap : 1);
  if (cudaMalloc(&drp, 8 * (n_rays + 1)) != cudaSuccess || cudaMalloc(&dcol, 4 * cap) != cudaSuccess ||
      cudaMalloc(&dval, 8 * cap) != cudaSuccess) {
    cudaFree(drp);
    cudaFree(dcol);
    cudaFree(dval);
    free_all(al);
    return fail(ctx, DP_ERR_ALLOC, "device allocation failed");
  }
  al.push_back(drp);
  al.push_back(dcol);
  al.push_back(dval);
  rc = tomo_core(ctx, P, n_rays, d.rays, d.rho, d.nE, d.nq, d.nw, d.flux, nullptr, nullptr, drp, dcol,
                 dval, nnz_cap, nnz);
  if (!rc) {
    cudaMemcpy(flux, d.flux, 8 * n_rays, cudaMemcpyDeviceToHost);
    cudaMemcpy(row_ptr, drp, 8 * (n_rays + 1), cudaMemcpyDeviceToHost);
    if (col) cudaMemcpy(col, dcol, 4 * size_t(*nnz), cudaMemcpyDeviceToHost);
    if (val) cudaMemcpy(val, dval, 8 * size_t(*nnz), cudaMemcpyDeviceToHost);
  }
  free_all(al);
  return rc;
}

int dp_tomo_vjp(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr, const dp_tomo_params* tp,
                const double* rho, long n_rays, const dp_ray* rays, const double* cot, double* flux,
                double* grad) {
  if (!flux || !cot || !grad || n_rays <= 0) return fail(ctx, DP_ERR_ARG, "bad output arrays");
  TomoDev P;
  std::vector<void*> al;
  HostTomo d{};
  int rc = upload_common(ctx, ph, gr, tp, rho, n_rays, rays, P, al, d);
  long ncell = long(gr->nx) * gr->ny * gr->nz;
  double *dcot = nullptr, *dgrad = nullptr;
  if (!rc) {
    if (cudaMalloc(&dcot, 8 * n_rays) != cudaSuccess || cudaMalloc(&dgrad, 8 * ncell) != cudaSuccess)
      rc = fail(ctx, DP_ERR_ALLOC, "device allocation failed");
    al.push_back(dcot);
    al.push_back(dgrad);
  }
  if (!rc && cudaMemcpy(dcot, cot, 8 * n_rays, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = fail(ctx, DP_ERR_CUDA, "cotangent upload failed");
  if (!rc)
    rc = tomo_core(ctx, P, n_rays, d.rays, d.rho, d.nE, d.nq, d.nw, d.flux, dcot, dgrad, nullptr,
                   nullptr, nullptr, 0, nullptr);
  if (!rc) {
    cudaMemcpy(flux, d.flux, 8 * n_rays, cudaMemcpyDeviceToHost);
    cudaMemcpy(grad, dgrad, 8 * ncell, cudaMemcpyDeviceToHost);
  }
  free_all(al);
  return rc;
}

int dp_tomo_forward_plain_dev(dp_ctx* ctx, const dp_physics* ph, const dp_grid* gr,
                              const dp_tomo_params* tp, const double* rho, long n_rays,
                              const dp_ray* rays, double* flux) {
  TomoDev P;
  int rc = make_params(ctx, ph, gr, tp, P);
  if (rc) return rc;
  if (tp->n_nodes > 1024) return fail(ctx, DP_ERR_ARG, "plain form supports up to 1024 nodes");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  double* part = static_cast<double*>(scratch(ctx, size_t(n_rays) * tp->n_nodes * 8));
  if (!part) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  P.rays = rays;
  P.n_rays = n_rays;
  P.rho = rho;
  P.nE = tp->node_energy;
  P.nq = tp->node_charge;
  P.nw = tp->node_weight;
  P.val = part;
  for (long r = 0; r < n_rays; ++r) plain_ray_kernel<<<1, tp->n_nodes, 0, ctx->stream>>>(P, r);
  plain_sum_kernel<<<int((n_rays + 127) / 128), 128, 0, ctx->stream>>>(part, n_rays, tp->n_nodes, flux);
  ctx->launches += n_rays + 1;
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  return check(ctx);
}

}  // extern "C"

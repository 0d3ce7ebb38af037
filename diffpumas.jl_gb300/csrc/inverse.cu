// inverse.cu -- inversion loops on the device over resident ray paths, the
// consumers of the tomography forward model and its Jacobian
// (src/Tomography_inverse.jl):
//
//   SART  (:98-132)  rho <- clamp(rho + lambda D_col J^T D_row (obs - f(rho)), box)
//                    with D_row = 1/sum_j|J_ij|, D_col = 1/sum_i|J_ij|; the
//                    Jacobian is re-evaluated at every iterate (the reference
//                    solves a fixed linear system A w = b).
//   Gauss-Newton (:448-603, legacy acceptance) on 0.5 sum_i W_i (f_i - obs_i)^2:
//                    the Levenberg-Marquardt system (J^T W J + mu diag) d = -g
//                    is solved matrix-free by Jacobi-preconditioned conjugate
//                    gradients (J v and J^T u on the CSR/CSC layouts) instead
//                    of a dense normal matrix, then a backtracking line search
//                    with the reference's acceptance f_new < f - 1e-10 |f|.
//
// The unknown is the voxel density (the reference's water fraction w maps
// onto it linearly).  All reductions run in a fixed order (deterministic).
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace dp {
namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 304;  // 2 x 152 SMs for the reduction partials

// y_i = sum_j J_ij x_j over the row's cells (side-exit entries excluded);
// one warp per row.
template <class V>
__global__ void spmv_kernel(const int64_t* row_ptr, const int32_t* cell, const V* val,
                            const double* x, long n_rows, const double* wt, double* y) {
  long r = (blockIdx.x * long(blockDim.x) + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (r >= n_rows) return;
  double s = 0.0;
  for (int64_t p = row_ptr[r] + lane, e = row_ptr[r + 1]; p < e; p += 32) {
    int c = cell[p];
    if (c >= 0) s += double(val[p]) * x[c];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[r] = wt ? wt[r] * s : s;
}

// Row sums of |J| (SART's D_row; zero rows count as 1).
template <class V>
__global__ void rowabs_kernel(const int64_t* row_ptr, const int32_t* cell, const V* val,
                              long n_rows, double* out) {
  long r = (blockIdx.x * long(blockDim.x) + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (r >= n_rows) return;
  double s = 0.0;
  for (int64_t p = row_ptr[r] + lane, e = row_ptr[r + 1]; p < e; p += 32)
    if (cell[p] >= 0) s += fabs(double(val[p]));
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[r] = s > 0.0 ? s : 1.0;
}

// Column sums over the CSC buckets: mode 0 sum_i |J_ij| (SART's D_col, zero
// columns count as 1); mode 1 sum_i W_i J_ij^2 (the Gauss-Newton diagonal).
// A ray can cross a cell in several segments: J_ij is the sum of its
// segments' entries, which sit next to each other in the bucket (ordered by
// entry index), so runs of one row are merged before squaring.
// One thread per cell with at most kBigBucket entries; the larger buckets
// (the cells next to a detector, crossed by thousands of rays) go to
// colsum_big_kernel.
constexpr int kBigBucket = 32;  // the bucket split of the J^T v gather (tomo.cu)
template <class V>
__global__ void colsum_kernel(const int64_t* cptr, const int32_t* perm, const V* val,
                              const int32_t* prow, const double* wt, long ncell, int mode,
                              double* out) {
  long c = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (c >= ncell) return;
  if (cptr[c + 1] - cptr[c] > kBigBucket) return;
  double s = 0.0, run = 0.0;
  int row = -1;
  for (int64_t p = cptr[c], e = cptr[c + 1]; p < e; ++p) {
    const int r = prow[p];
    if (r != row) {
      if (row >= 0) s += mode == 0 ? fabs(run) : (wt ? wt[row] : 1.0) * run * run;
      row = r;
      run = 0.0;
    }
    run += double(val[perm ? perm[p] : p]);
  }
  if (row >= 0) s += mode == 0 ? fabs(run) : (wt ? wt[row] : 1.0) * run * run;
  out[c] = mode == 0 ? (s > 0.0 ? s : 1.0) : s;
}
// A block of kBigThreads per large bucket: the bucket is cut into
// kBigThreads contiguous chunks and each run of one row belongs to the thread
// whose chunk it starts in (a thread skips the tail of the run entering its
// chunk and finishes its last run past the chunk end), so every run is merged
// before squaring, as above; the threads' sums combine in a fixed order.
template <class V>
__global__ void __launch_bounds__(kBigThreads) colsum_big_kernel(
    const int64_t* cptr, const int32_t* perm, const V* val, const int32_t* prow,
    const double* wt, const int32_t* big, int mode, double* out) {
  __shared__ double sh[kBigThreads / 32];
  const int c = big[blockIdx.x];
  const int64_t b = cptr[c], e = cptr[c + 1];
  const int64_t len = (e - b + kBigThreads - 1) / kBigThreads;
  int64_t p = b + threadIdx.x * len;
  const int64_t stop = p + len < e ? p + len : e;
  double s = 0.0;
  if (p < stop) {
    if (p > b) {
      const int prev = prow[p - 1];
      while (p < stop && prow[p] == prev) ++p;
    }
    while (p < stop) {
      const int r = prow[p];
      double run = 0.0;
      for (; p < e && prow[p] == r; ++p) run += double(val[perm ? perm[p] : p]);
      s += mode == 0 ? fabs(run) : (wt ? wt[r] : 1.0) * run * run;
    }
  }
  s = big_block_sum(s, sh);
  if (threadIdx.x == 0) out[c] = mode == 0 ? (s > 0.0 ? s : 1.0) : s;
}

// Fixed-order dot product: block partials, then one block.
__global__ void __launch_bounds__(kThreads) dot_part_kernel(const double* a, const double* b,
                                                            const double* w, long n, double* part) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (long i = blockIdx.x * long(kThreads) + threadIdx.x; i < n; i += long(gridDim.x) * kThreads) {
    double v = a[i] * (b ? b[i] : a[i]);
    s += w ? w[i] * v : v;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void __launch_bounds__(kThreads) dot_final_kernel(const double* part, int nb,
                                                             double* out) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += kThreads) s += part[b];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// r_i = s (f_i - obs_i); with wr: wr_i = W_i r_i as well.
__global__ void residual_kernel(const double* f, const double* obs, const double* wt, long n,
                                double sgn, double* r, double* wr) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x) {
    double v = sgn * (f[i] - obs[i]);
    r[i] = v;
    if (wr) wr[i] = (wt ? wt[i] : 1.0) * v;
  }
}
// u_i = a_i / b_i
__global__ void divide_kernel(const double* a, const double* b, long n, double* u) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    u[i] = a[i] / b[i];
}
// SART update: rho = clamp(rho + lambda g / colsum, box)
__global__ void sart_update_kernel(double* rho, const double* g, const double* colsum, long n,
                                   double lambda, double lo, double hi) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    rho[i] = fmin(fmax(rho[i] + lambda * g[i] / colsum[i], lo), hi);
}

// Conjugate-gradient pieces with device-resident scalars (no host round trip
// inside the CG loop).  s[0] = r.z, s[1] = p.Ap, s[2] = new r.z.
__global__ void cg_init_kernel(const double* g, const double* prec, long n, double* x, double* r,
                               double* z, double* p) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x) {
    double ri = -g[i];
    double zi = ri / prec[i];
    x[i] = 0.0;
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
  }
}
// trial = clamp(rho + alpha d, box)
__global__ void trial_kernel(const double* rho, const double* d, long n, double alpha, double lo,
                             double hi, double* out) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    out[i] = fmin(fmax(rho[i] + alpha * d[i], lo), hi);
}
// prec = max(diag, floor) (Jacobi preconditioner) and damp = mu max(diag, floor)
__global__ void lm_diag_kernel(const double* diag, long n, double floor_, double mu, double* prec,
                               double* damp) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x) {
    double d = fmax(diag[i], floor_);
    damp[i] = mu * d;
    prec[i] = (1.0 + mu) * d;
  }
}
__global__ void max_part_kernel(const double* a, long n, double* part) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (long i = blockIdx.x * long(kThreads) + threadIdx.x; i < n; i += long(gridDim.x) * kThreads)
    s = fmax(s, a[i]);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Smoothness prior on the voxel grid's 6-neighbour graph (SmoothnessPrior,
// src/Tomography_inverse.jl:17-79, 262-268): R = weight sum_edges (x_i - x_j)^2.
struct Dims {
  int nx, ny, nz;
};
__device__ __forceinline__ int degree(Dims d, long c, int* nb) {
  const long sxy = long(d.nx) * d.ny;
  const int i = int(c % d.nx), j = int((c / d.nx) % d.ny), k = int(c / sxy);
  int n = 0;
  if (i > 0) nb[n++] = int(c - 1);
  if (i < d.nx - 1) nb[n++] = int(c + 1);
  if (j > 0) nb[n++] = int(c - d.nx);
  if (j < d.ny - 1) nb[n++] = int(c + d.nx);
  if (k > 0) nb[n++] = int(c - sxy);
  if (k < d.nz - 1) nb[n++] = int(c + sxy);
  return n;
}
// sum_{j in N(c)} (x_c - x_j), neighbours in the order of degree(): -x, +x,
// -y, +y, -z, +z (no neighbour array, so nothing goes to local memory)
__device__ __forceinline__ double lap_sum(const double* x, Dims d, long c) {
  const long sxy = long(d.nx) * d.ny;
  const long k = c / sxy, rem = c - k * sxy;
  const int j = int(rem / d.nx), i = int(rem - long(j) * d.nx);
  const double xc = x[c];
  double s = 0.0;
  if (i > 0) s += xc - x[c - 1];
  if (i < d.nx - 1) s += xc - x[c + 1];
  if (j > 0) s += xc - x[c - d.nx];
  if (j < d.ny - 1) s += xc - x[c + d.nx];
  if (k > 0) s += xc - x[c - sxy];
  if (k < d.nz - 1) s += xc - x[c + sxy];
  return s;
}
// out = (accumulate ? out : 0) + coef * sum_{j in N(c)} (x_c - x_j)
__global__ void lap_kernel(const double* x, Dims d, double coef, int accumulate, double* out) {
  const long n = long(d.nx) * d.ny * d.nz;
  for (long c = blockIdx.x * long(blockDim.x) + threadIdx.x; c < n;
       c += long(gridDim.x) * blockDim.x)
    out[c] = (accumulate ? out[c] : 0.0) + coef * lap_sum(x, d, c);
}
__device__ __forceinline__ void block_part(double s, double* sh, double* part) {
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
// CG operator tail in one pass: Ap += damp p (+ coef L p when coef != 0),
// and the block partials of p . Ap in dot_part_kernel's traversal
// (kRedBlocks blocks, grid stride), finished by dot_final_kernel.
__global__ void __launch_bounds__(kThreads) cg_apply_kernel(const double* p, const double* damp,
                                                            Dims d, double coef, long n,
                                                            double* Ap, double* part) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (long i = blockIdx.x * long(kThreads) + threadIdx.x; i < n; i += long(gridDim.x) * kThreads) {
    const double pi = p[i];
    double t = Ap[i] + damp[i] * pi;
    if (coef != 0.0) t = t + coef * lap_sum(p, d, i);
    Ap[i] = t;
    s += pi * t;
  }
  block_part(s, sh, part);
}
// x += a p, r -= a Ap, z = r / prec with a = s[0] / s[1], and the block
// partials of r . z (same traversal as above).
__global__ void __launch_bounds__(kThreads) cg_step_dot_kernel(const double* s, const double* p,
                                                               const double* Ap,
                                                               const double* prec, long n,
                                                               double* x, double* r, double* z,
                                                               double* part) {
  __shared__ double sh[kThreads];
  const double a = s[1] != 0.0 ? s[0] / s[1] : 0.0;
  double acc = 0.0;
  for (long i = blockIdx.x * long(kThreads) + threadIdx.x; i < n; i += long(gridDim.x) * kThreads) {
    x[i] += a * p[i];
    const double ri = r[i] - a * Ap[i];
    r[i] = ri;
    const double zi = ri / prec[i];
    z[i] = zi;
    acc += ri * zi;
  }
  block_part(acc, sh, part);
}
// r . z from the partials: s[2] = it, s[5] = s[2] / s[0] (0 if s[0] is 0,
// the CG beta), then s[0] = s[2].
__global__ void __launch_bounds__(kThreads) cg_beta_kernel(const double* part, int nb, double* s) {
  __shared__ double sh[kThreads];
  double v = 0.0;
  for (int b = threadIdx.x; b < nb; b += kThreads) v += part[b];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double rz = sh[0];
    s[2] = rz;
    s[5] = s[0] != 0.0 ? rz / s[0] : 0.0;
    s[0] = rz;
  }
}
// p = z + beta p with beta = s[5]
__global__ void cg_dir_beta_kernel(const double* s, const double* z, long n, double* p) {
  const double b = s[5];
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    p[i] = z[i] + b * p[i];
}
// block partials of sum over the forward edges of (x_i - x_j)^2
__global__ void __launch_bounds__(kThreads) prior_part_kernel(const double* x, Dims d,
                                                              double* part) {
  __shared__ double sh[kThreads];
  const long n = long(d.nx) * d.ny * d.nz, sxy = long(d.nx) * d.ny;
  double s = 0.0;
  for (long c = blockIdx.x * long(kThreads) + threadIdx.x; c < n;
       c += long(gridDim.x) * kThreads) {
    const int i = int(c % d.nx), j = int((c / d.nx) % d.ny), k = int(c / sxy);
    if (i < d.nx - 1) s += (x[c] - x[c + 1]) * (x[c] - x[c + 1]);
    if (j < d.ny - 1) s += (x[c] - x[c + d.nx]) * (x[c] - x[c + d.nx]);
    if (k < d.nz - 1) s += (x[c] - x[c + sxy]) * (x[c] - x[c + sxy]);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
// diag += coef * degree (the prior Hessian's diagonal)
__global__ void add_degree_kernel(Dims d, double coef, double* diag) {
  const long n = long(d.nx) * d.ny * d.nz;
  for (long c = blockIdx.x * long(blockDim.x) + threadIdx.x; c < n;
       c += long(gridDim.x) * blockDim.x) {
    int nb[6];
    diag[c] += coef * degree(d, c, nb);
  }
}
// one smoothing sweep (apply_laplacian_smoothing, :64-79), then the box
__global__ void smooth_kernel(const double* x, Dims d, double strength, double lo, double hi,
                              double* out) {
  const long n = long(d.nx) * d.ny * d.nz;
  for (long c = blockIdx.x * long(blockDim.x) + threadIdx.x; c < n;
       c += long(gridDim.x) * blockDim.x) {
    int nb[6];
    const int m = degree(d, c, nb);
    double mean = 0.0;
    for (int t = 0; t < m; ++t) mean += x[nb[t]];
    double v = m ? (1.0 - strength) * x[c] + strength * (mean / m) : x[c];
    out[c] = fmin(fmax(v, lo), hi);
  }
}

// ---- MLEM on the model linearised at an iterate (A = -J >= 0, b = f + A rho - obs)
__global__ void fill_kernel(double* a, long n, double v) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    a[i] = v;
}
// a = clamp(max(a, floor), lo, hi)
__global__ void clamp_kernel(double* a, long n, double floor_, double lo, double hi) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    a[i] = fmin(fmax(fmax(a[i], floor_), lo), hi);
}
// b0 = max(f + A rho - obs, 0) with A rho = -y (y = J rho)
__global__ void mlem_rhs_kernel(const double* y, const double* f, const double* obs, long n,
                                double* b0) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    b0[i] = fmax(f[i] - y[i] - obs[i], 0.0);
}
// ratio = b / max(A rho, 1e-12), b = b0 (fixed linearisation) or max(f + A rho - obs, 0)
__global__ void mlem_ratio_kernel(const double* y, const double* f, const double* obs,
                                  const double* b0, long n, double* ratio) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x) {
    const double aw = -y[i];
    const double b = b0 ? b0[i] : fmax(f[i] + aw - obs[i], 0.0);
    ratio[i] = b / fmax(aw, 1e-12);
  }
}
// rho <- clamp(rho * A^T ratio / (A^T 1 + max(pg, 0)), box), A^T v = -J^T v; a
// column sum A^T 1 <= 0 counts as 1 (mlem_reconstruct's sens)
__global__ void mlem_update_kernel(double* rho, const double* jt_ratio, const double* jt_one,
                                   const double* pg, long n, double lo, double hi) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x) {
    double sens = -jt_one[i];
    if (sens <= 0.0) sens = 1.0;
    const double den = sens + (pg ? fmax(pg[i], 0.0) : 0.0);
    rho[i] = fmin(fmax(rho[i] * (-jt_ratio[i]) / den, lo), hi);
  }
}
// ---- gradient descent
// p = g / max(d, floor) (PGD's preconditioned direction)
__global__ void precond_kernel(const double* g, const double* d, long n, double floor_, double* p) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    p[i] = g[i] / fmax(d[i], floor_);
}
// Adam (beta1 0.9, beta2 0.999, eps 1e-8) with bias corrections c1 = 1 - 0.9^t,
// c2 = 1 - 0.999^t, then the box
__global__ void adam_kernel(double* w, const double* g, double* m, double* v, long n, double lr,
                            double c1, double c2, double lo, double hi) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x) {
    const double gi = g[i];
    const double mi = 0.9 * m[i] + (1.0 - 0.9) * gi;
    const double vi = 0.999 * v[i] + (1.0 - 0.999) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] = fmin(fmax(w[i] - lr * (mi / c1) / (sqrt(vi / c2) + 1e-8), lo), hi);
  }
}
// out = a - b
__global__ void sub_kernel(const double* a, const double* b, long n, double* out) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    out[i] = a[i] - b[i];
}
// out += a
__global__ void add_kernel(const double* a, long n, double* out) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n;
       i += long(gridDim.x) * blockDim.x)
    out[i] += a[i];
}

struct Solver {
  dp_ctx* ctx;
  const dp_physics* ph;
  const dp_paths* pa;
  const dp_tomo_params* tp;
  int precision;
  long n_rays, ncell;
  void* jv;      // Jacobian values (FP32 or FP64), CSR (segment) order
  void* jcsc;    // the same values in CSC (bucket) order, for J^T v and column sums
  double* part;  // reduction partials
  double* s;     // device scalars
  int grid(long n) const { return int(std::min<long>((n + kThreads - 1) / kThreads, 152L * 8)); }

  int dot(const double* a, const double* b, const double* w, long n, double* out) {
    timed_begin(ctx);
    dot_part_kernel<<<kRedBlocks, kThreads, 0, ctx->stream>>>(a, b, w, n, part);
    dot_final_kernel<<<1, kThreads, 0, ctx->stream>>>(part, kRedBlocks, out);
    ++ctx->launches;  // the second of the pair (timed_begin counts the first)
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "gn_dot");
    return DP_OK;
  }
  // the CG operator tail and step, each with its reduction (timed with the dots)
  int cg_apply(const double* p, const double* damp, double coef, long n, double* Ap) {
    timed_begin(ctx);
    cg_apply_kernel<<<kRedBlocks, kThreads, 0, ctx->stream>>>(p, damp, dims, coef, n, Ap, part);
    dot_final_kernel<<<1, kThreads, 0, ctx->stream>>>(part, kRedBlocks, s + 1);
    ++ctx->launches;
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "gn_cg");
    return DP_OK;
  }
  int cg_step(const double* p, const double* Ap, const double* prec, long n, double* x, double* r,
              double* z) {
    timed_begin(ctx);
    cg_step_dot_kernel<<<kRedBlocks, kThreads, 0, ctx->stream>>>(s, p, Ap, prec, n, x, r, z, part);
    cg_beta_kernel<<<1, kThreads, 0, ctx->stream>>>(part, kRedBlocks, s);
    ++ctx->launches;
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "gn_cg");
    return DP_OK;
  }
  double host_scalar(const double* d) {
    double h = 0.0;
    cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return h;
  }
  int spmv(const double* x, const double* wt, double* y) {
    int blocks = int((n_rays * 32 + kThreads - 1) / kThreads);
    timed_begin(ctx);
    if (precision)
      spmv_kernel<float><<<blocks, kThreads, 0, ctx->stream>>>(pa->row_ptr, pa->cell,
                                                               static_cast<const float*>(jv), x,
                                                               n_rays, wt, y);
    else
      spmv_kernel<double><<<blocks, kThreads, 0, ctx->stream>>>(pa->row_ptr, pa->cell,
                                                                static_cast<const double*>(jv), x,
                                                                n_rays, wt, y);
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "gn_spmv");
    return DP_OK;
  }
  int transpose(const double* u, double* out) {
    return tomo_transpose(ctx, pa, jcsc, precision, u, out, true);
  }
  int colsum(const double* wt, int mode, double* out) {
    int blocks = int((ncell + kThreads - 1) / kThreads);
    timed_begin(ctx);
    if (precision) {
      const float* v = static_cast<const float*>(jcsc);
      colsum_kernel<float><<<blocks, kThreads, 0, ctx->stream>>>(pa->cptr, nullptr, v, pa->prow,
                                                                 wt, ncell, mode, out);
      if (pa->n_big > 0)
        colsum_big_kernel<float><<<pa->n_big, kBigThreads, 0, ctx->stream>>>(
            pa->cptr, nullptr, v, pa->prow, wt, pa->big, mode, out);
    } else {
      const double* v = static_cast<const double*>(jcsc);
      colsum_kernel<double><<<blocks, kThreads, 0, ctx->stream>>>(pa->cptr, nullptr, v, pa->prow,
                                                                  wt, ncell, mode, out);
      if (pa->n_big > 0)
        colsum_big_kernel<double><<<pa->n_big, kBigThreads, 0, ctx->stream>>>(
            pa->cptr, nullptr, v, pa->prow, wt, pa->big, mode, out);
    }
    if (pa->n_big > 0) ++ctx->launches;
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    timed_end(ctx, "gn_colsum");
    return DP_OK;
  }
  int rowabs(double* out) {
    int blocks = int((n_rays * 32 + kThreads - 1) / kThreads);
    if (precision)
      rowabs_kernel<float><<<blocks, kThreads, 0, ctx->stream>>>(
          pa->row_ptr, pa->cell, static_cast<const float*>(jv), n_rays, out);
    else
      rowabs_kernel<double><<<blocks, kThreads, 0, ctx->stream>>>(
          pa->row_ptr, pa->cell, static_cast<const double*>(jv), n_rays, out);
    ++ctx->launches;
    DP_CHECK_CUDA(ctx, cudaGetLastError());
    return DP_OK;
  }
  // forward (and Jacobian when jac) at rho
  int eval(const double* rho, double* flux, bool jac) {
    const int rc = tomo_eval_raw(ctx, ph, pa, tp, rho, flux, jac ? jv : nullptr, precision);
    if (rc || !jac) return rc;
    return tomo_csc_values(ctx, pa, jv, precision, jcsc);
  }
  Dims dims;
  double prior = 0.0;  // smoothness weight
  // 0.5 sum W (f - obs)^2 + prior(rho), on the host
  double objective(const double* f, const double* obs, const double* wt, double* r,
                   const double* rho) {
    residual_kernel<<<grid(n_rays), kThreads, 0, ctx->stream>>>(f, obs, wt, n_rays, 1.0, r,
                                                               nullptr);
    ++ctx->launches;
    dot(r, r, wt, n_rays, s + 3);
    if (prior > 0.0) {
      prior_part_kernel<<<kRedBlocks, kThreads, 0, ctx->stream>>>(rho, dims, part);
      dot_final_kernel<<<1, kThreads, 0, ctx->stream>>>(part, kRedBlocks, s + 4);
      ctx->launches += 2;
    }
    double v = 0.5 * host_scalar(s + 3);
    if (prior > 0.0) v += prior * host_scalar(s + 4);
    return v;
  }
};

}  // namespace
}  // namespace dp

using namespace dp;

extern "C" {

int dp_tomo_solve_dev(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa,
                      const dp_tomo_params* tp, const double* obs, const double* weight,
                      double* rho, const dp_solve_params* sp, double* history) {
  if (!ctx || !ph || !pa || !tp || !obs || !rho || !sp)
    return fail(ctx, DP_ERR_ARG, "null argument");
  if (sp->n_iter < 0 || sp->method < DP_SOLVE_SART || sp->method > DP_SOLVE_GD ||
      sp->optimizer < DP_GD_PGD || sp->optimizer > DP_GD_PLAIN ||
      (sp->precision != DP_PREC_FP64 && sp->precision != DP_PREC_MIXED) ||
      !(sp->box_hi > sp->box_lo))
    return fail(ctx, DP_ERR_ARG, "invalid solver parameters");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  Solver S{};
  S.ctx = ctx;
  S.ph = ph;
  S.pa = pa;
  S.tp = tp;
  S.precision = sp->precision;
  S.n_rays = pa->n_rays;
  S.ncell = long(pa->grid.nx) * pa->grid.ny * pa->grid.nz;
  S.dims = Dims{pa->grid.nx, pa->grid.ny, pa->grid.nz};
  S.prior = sp->prior_weight > 0.0 ? sp->prior_weight : 0.0;
  const long nr = S.n_rays, nc = S.ncell;
  // slot 0: Jacobian values (CSR and CSC order), 5 row vectors, 10 cell vectors,
  // partials, scalars
  size_t need = 2 * size_t(pa->nnz + 1) * (S.precision ? 4 : 8) + size_t(nr) * 5 * 8 +
                size_t(nc) * 10 * 8 + kRedBlocks * 8 + 64 + 16 * 256;
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, need, 0));
  A.cap = ctx->slot_bytes[0];
  S.jv = A.take<char>(size_t(pa->nnz + 1) * (S.precision ? 4 : 8));
  S.jcsc = A.take<char>(size_t(pa->nnz + 1) * (S.precision ? 4 : 8));
  double *flux = A.take<double>(nr), *r = A.take<double>(nr), *u = A.take<double>(nr),
         *rowsum = A.take<double>(nr), *tmp = A.take<double>(nr);
  double *g = A.take<double>(nc), *col = A.take<double>(nc), *x = A.take<double>(nc),
         *cr = A.take<double>(nc), *z = A.take<double>(nc), *p = A.take<double>(nc),
         *Ap = A.take<double>(nc), *prec = A.take<double>(nc), *damp = A.take<double>(nc),
         *trial = A.take<double>(nc);
  S.part = A.take<double>(kRedBlocks);
  S.s = A.take<double>(8);
  if (!S.s) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  const int saved = ctx->blocking;
  ctx->blocking = 0;  // kernels are enqueued; host reads only the line-search scalars
  int rc = DP_OK;
  if (history)
    for (int k = 0; k <= sp->n_iter; ++k) history[k] = std::nan("");
  auto record = [&](int k, double v) {
    if (history) history[k] = v;
  };
  if (sp->method == DP_SOLVE_SART) {
    const double lambda = sp->relaxation > 0.0 ? sp->relaxation : 0.2;
    for (int it = 0; it < sp->n_iter && !rc; ++it) {
      rc = S.eval(rho, flux, true);
      if (rc) break;
      residual_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(flux, obs, nullptr, nr, -1.0, r,
                                                                 nullptr);
      ++ctx->launches;
      S.dot(r, r, nullptr, nr, S.s + 3);
      record(it, std::sqrt(S.host_scalar(S.s + 3)));
      if ((rc = S.rowabs(rowsum))) break;
      divide_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(r, rowsum, nr, u);
      ++ctx->launches;
      if ((rc = S.transpose(u, g))) break;
      if ((rc = S.colsum(nullptr, 0, col))) break;
      sart_update_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, g, col, nc, lambda,
                                                                   sp->box_lo, sp->box_hi);
      ++ctx->launches;
      if (S.prior > 0.0) {  // smoothing sweep of the Tikhonov-style prior
        const double strength = sp->smooth_strength > 0.0 ? sp->smooth_strength : 0.1;
        smooth_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, S.dims, strength, sp->box_lo,
                                                                sp->box_hi, trial);
        DP_CHECK_CUDA(ctx, cudaMemcpyAsync(rho, trial, nc * 8, cudaMemcpyDeviceToDevice,
                                           ctx->stream));
        ++ctx->launches;
      }
    }
  } else if (sp->method == DP_SOLVE_MLEM) {
    // mlem_reconstruct (src/Tomography_inverse.jl:153-188) with A = -J, b = f + A rho - obs
    const bool fixed = sp->fixed_linearization != 0;
    double *ratio = rowsum, *b0 = u, *jt_one = prec, *back = g, *pg = Ap;
    clamp_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, nc, 1e-6, -1e300, 1e300);
    ++ctx->launches;
    for (int it = 0; it < sp->n_iter && !rc; ++it) {
      if ((rc = S.eval(rho, flux, it == 0 || !fixed))) break;
      residual_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(flux, obs, nullptr, nr, -1.0, r,
                                                                 nullptr);
      ++ctx->launches;
      S.dot(r, r, nullptr, nr, S.s + 3);
      record(it, std::sqrt(S.host_scalar(S.s + 3)));
      if (it == 0 || !fixed) {
        fill_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(tmp, nr, 1.0);
        ++ctx->launches;
        if ((rc = S.transpose(tmp, jt_one))) break;  // J^T 1
      }
      if ((rc = S.spmv(rho, nullptr, r))) break;  // y = J rho
      if (fixed && it == 0) {
        mlem_rhs_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(r, flux, obs, nr, b0);
        ++ctx->launches;
      }
      mlem_ratio_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(r, flux, obs,
                                                                  fixed ? b0 : nullptr, nr, ratio);
      ++ctx->launches;
      if ((rc = S.transpose(ratio, back))) break;  // J^T ratio
      if (S.prior > 0.0) {
        lap_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, S.dims, 2.0 * S.prior, 0, pg);
        ++ctx->launches;
      }
      mlem_update_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(
          rho, back, jt_one, S.prior > 0.0 ? pg : nullptr, nc, sp->box_lo, sp->box_hi);
      ++ctx->launches;
      DP_CHECK_CUDA(ctx, cudaGetLastError());
    }
  } else if (sp->method == DP_SOLVE_GD) {
    // gradient_descent_reconstruct (src/Tomography_inverse.jl:324-400)
    const bool fixed = sp->fixed_linearization != 0;
    const int opt = sp->optimizer;
    const double lr = sp->lr > 0.0 ? sp->lr : (opt == DP_GD_PGD ? 1.0 : 1e-2);
    double *f0 = rowsum, *rho0 = x, *m = cr, *v = z, *dir = p, *lp = Ap, *diag = col;
    clamp_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, nc, -1e300, sp->box_lo,
                                                           sp->box_hi);
    ++ctx->launches;
    rc = S.eval(rho, flux, true);
    if (!rc && fixed) {
      DP_CHECK_CUDA(ctx, cudaMemcpyAsync(f0, flux, nr * 8, cudaMemcpyDeviceToDevice, ctx->stream));
      DP_CHECK_CUDA(ctx, cudaMemcpyAsync(rho0, rho, nc * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    if (opt == DP_GD_ADAM) {
      DP_CHECK_CUDA(ctx, cudaMemsetAsync(m, 0, nc * 8, ctx->stream));
      DP_CHECK_CUDA(ctx, cudaMemsetAsync(v, 0, nc * 8, ctx->stream));
    }
    double prev = rc ? 0.0 : S.objective(flux, obs, weight, r, rho);
    if (!rc) {
      S.dot(r, r, nullptr, nr, S.s + 3);
      record(0, std::sqrt(S.host_scalar(S.s + 3)));
    }
    double c1 = 1.0, c2 = 1.0;
    for (int t = 1; t <= sp->n_iter && !rc; ++t) {
      // g = J^T W (pred - obs) + dR/drho
      residual_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(flux, obs, weight, nr, 1.0, r, u);
      ++ctx->launches;
      if ((rc = S.transpose(u, g))) break;
      if (S.prior > 0.0) {
        lap_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, S.dims, 2.0 * S.prior, 1, g);
        ++ctx->launches;
      }
      if (opt == DP_GD_PGD) {
        // Jacobi (Gauss-Newton + prior) preconditioner and the exact step length
        // of the local quadratic along p = D^-1 g, capped at lr
        if ((rc = S.colsum(weight, 1, diag))) break;
        if (S.prior > 0.0) {
          add_degree_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(S.dims, 2.0 * S.prior, diag);
          ++ctx->launches;
        }
        max_part_kernel<<<kRedBlocks, kThreads, 0, ctx->stream>>>(diag, nc, S.part);
        ++ctx->launches;
        std::vector<double> hp(kRedBlocks);
        DP_CHECK_CUDA(ctx, cudaMemcpyAsync(hp.data(), S.part, kRedBlocks * 8,
                                           cudaMemcpyDeviceToHost, ctx->stream));
        DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        double dmax = 0.0;
        for (double hv : hp) dmax = std::max(dmax, hv);
        if (!(dmax > 0.0)) dmax = 1.0;
        precond_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(g, diag, nc, 1e-9 * dmax, dir);
        ++ctx->launches;
        if ((rc = S.spmv(dir, nullptr, tmp))) break;  // J p
        S.dot(tmp, tmp, weight, nr, S.s + 3);         // p^T J^T W J p
        S.dot(g, dir, nullptr, nc, S.s + 4);          // g . p
        double denom = S.host_scalar(S.s + 3);
        const double num = S.host_scalar(S.s + 4);
        if (S.prior > 0.0) {
          lap_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(dir, S.dims, 2.0 * S.prior, 0, lp);
          ++ctx->launches;
          S.dot(dir, lp, nullptr, nc, S.s + 5);
          denom += S.host_scalar(S.s + 5);
        }
        const double alpha =
            (denom > 0.0 && std::isfinite(num)) ? std::min(std::max(num / denom, 0.0), lr) : 0.0;
        trial_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, dir, nc, -alpha, sp->box_lo,
                                                               sp->box_hi, rho);
        ++ctx->launches;
      } else if (opt == DP_GD_ADAM) {
        c1 *= 0.9;
        c2 *= 0.999;
        adam_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, g, m, v, nc, lr, 1.0 - c1,
                                                              1.0 - c2, sp->box_lo, sp->box_hi);
        ++ctx->launches;
      } else {
        trial_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, g, nc, -lr, sp->box_lo,
                                                               sp->box_hi, rho);
        ++ctx->launches;
      }
      DP_CHECK_CUDA(ctx, cudaGetLastError());
      // the model at the new iterate: re-evaluated, or f0 + J0 (rho - rho0)
      if (!fixed) {
        if ((rc = S.eval(rho, flux, true))) break;
      } else {
        sub_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, rho0, nc, lp);
        ++ctx->launches;
        if ((rc = S.spmv(lp, nullptr, flux))) break;
        add_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(f0, nr, flux);
        ++ctx->launches;
      }
      const double obj = S.objective(flux, obs, weight, r, rho);
      S.dot(r, r, nullptr, nr, S.s + 3);
      record(t, std::sqrt(S.host_scalar(S.s + 3)));
      if (opt == DP_GD_PGD &&
          std::fabs(obj - prev) <= 1e-5 * std::max(std::fabs(prev), 2.220446049250313e-16))
        break;
      prev = obj;
    }
  } else {
    double mu = sp->lm_damping > 0.0 ? sp->lm_damping : 1e-3;
    const int cg_iter = sp->cg_iter > 0 ? sp->cg_iter : 10;
    rc = S.eval(rho, flux, true);
    double f_cur = rc ? 0.0 : S.objective(flux, obs, weight, r, rho);
    bool speculate = sp->no_speculation == 0;
    for (int it = 0; it < sp->n_iter && !rc; ++it) {
      {
        S.dot(r, r, nullptr, nr, S.s + 3);
        record(it, std::sqrt(S.host_scalar(S.s + 3)));
      }
      // gradient g = J^T W r and the Gauss-Newton diagonal sum_i W_i J_ij^2
      residual_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(flux, obs, weight, nr, 1.0, r, u);
      ++ctx->launches;
      if ((rc = S.transpose(u, g))) break;
      if ((rc = S.colsum(weight, 1, col))) break;
      if (S.prior > 0.0) {  // prior gradient 2 w L rho and Hessian diagonal 2 w deg
        lap_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, S.dims, 2.0 * S.prior, 1, g);
        add_degree_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(S.dims, 2.0 * S.prior, col);
        ctx->launches += 2;
      }
      max_part_kernel<<<kRedBlocks, kThreads, 0, ctx->stream>>>(col, nc, S.part);
      ++ctx->launches;
      std::vector<double> hp(kRedBlocks);
      DP_CHECK_CUDA(ctx, cudaMemcpyAsync(hp.data(), S.part, kRedBlocks * 8, cudaMemcpyDeviceToHost,
                                         ctx->stream));
      DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      double dmax = 0.0;
      for (double v : hp) dmax = std::max(dmax, v);
      if (!(dmax > 0.0)) dmax = 1.0;
      bool accepted = false, have_jac = false, first_trial = false;
      for (int attempt = 0; attempt < 6 && !accepted && !rc; ++attempt) {
        // (J^T W J + mu D) d = -g by Jacobi-preconditioned CG from d = 0
        lm_diag_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(col, nc, 1e-12 * dmax, mu, prec,
                                                                damp);
        cg_init_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(g, prec, nc, x, cr, z, p);
        ctx->launches += 2;
        S.dot(cr, z, nullptr, nc, S.s + 0);
        for (int k = 0; k < cg_iter && !rc; ++k) {
          if ((rc = S.spmv(p, weight, tmp))) break;  // W J p
          if ((rc = S.transpose(tmp, Ap))) break;    // J^T W J p
          // + mu D p (+ 2 w L p), and p . Ap
          if ((rc = S.cg_apply(p, damp, S.prior > 0.0 ? 2.0 * S.prior : 0.0, nc, Ap))) break;
          if ((rc = S.cg_step(p, Ap, prec, nc, x, cr, z))) break;  // r . z and beta
          cg_dir_beta_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(S.s, z, nc, p);
          ++ctx->launches;
        }
        if (rc) break;
        // backtracking line search, legacy acceptance (src/Tomography_inverse.jl:443-448)
        double alpha = 1.0;
        for (int ls = 0; ls < 14 && !rc; ++ls) {
          trial_kernel<<<S.grid(nc), kThreads, 0, ctx->stream>>>(rho, x, nc, alpha, sp->box_lo,
                                                                 sp->box_hi, trial);
          ++ctx->launches;
          // While full steps keep being accepted, the first trial is evaluated
          // with its Jacobian: on acceptance that is the next iteration's
          // Jacobian, on rejection the one at rho is rebuilt.
          const bool spec = speculate && attempt == 0 && ls == 0;
          if ((rc = S.eval(trial, tmp, spec))) break;
          double f_new = S.objective(tmp, obs, weight, u, trial);
          if (std::isfinite(f_new) && f_new < f_cur - 1e-10 * std::fabs(f_cur)) {
            DP_CHECK_CUDA(ctx, cudaMemcpyAsync(rho, trial, nc * 8, cudaMemcpyDeviceToDevice,
                                               ctx->stream));
            f_cur = f_new;
            accepted = true;
            have_jac = spec;
            first_trial = attempt == 0 && ls == 0;
            break;
          }
          if (spec && (rc = S.eval(rho, flux, true))) break;
          alpha *= 0.5;
        }
        if (accepted) mu = std::max(mu / 3.0, 1e-12);
        else mu = std::min(mu * 3.0, 1e12);
      }
      if (rc || !accepted) break;
      // speculate again in the next iteration only if this one took its
      // first trial (a halved or re-damped step predicts more rejections)
      speculate = sp->no_speculation == 0 && first_trial;
      if (have_jac) {  // flux, residual and Jacobian of the accepted trial are current
        DP_CHECK_CUDA(ctx, cudaMemcpyAsync(flux, tmp, nr * 8, cudaMemcpyDeviceToDevice,
                                           ctx->stream));
        DP_CHECK_CUDA(ctx, cudaMemcpyAsync(r, u, nr * 8, cudaMemcpyDeviceToDevice, ctx->stream));
      } else {
        rc = S.eval(rho, flux, true);
        if (!rc) f_cur = S.objective(flux, obs, weight, r, rho);
      }
    }
  }
  if (!rc && sp->method != DP_SOLVE_GD) {
    // final misfit ||obs - f(rho)|| (GD records every iterate itself, on the
    // model it iterates on)
    rc = S.eval(rho, flux, false);
    if (!rc) {
      residual_kernel<<<S.grid(nr), kThreads, 0, ctx->stream>>>(flux, obs, nullptr, nr, -1.0, r,
                                                                nullptr);
      ++ctx->launches;
      S.dot(r, r, nullptr, nr, S.s + 3);
      record(sp->n_iter, std::sqrt(S.host_scalar(S.s + 3)));
    }
  }
  ctx->blocking = saved;
  if (rc) return rc;
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return dp_sync(ctx);
}

}  // extern "C"

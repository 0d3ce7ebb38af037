// wtomo.cu -- the water-fraction CSDA forward model of src/Tomography.jl on
// the device: compute_directional_flux_csda (:667-727),
// directional_flux_and_grad_csda and assemble_forward_and_jacobian
// (:736-820), with the CSDA correction multipliers (:85-214, :367-412,
// :557-579).  Two instances of the walk (wtomo_walk.cuh): FP64, the
// reference's operations, and mixed precision, FP32 steps and tangents with
// the adjoint's prefix sums, the flux and the reductions in FP64.
//
// One warp per direction, one lane per energy sample.  d flux / d w comes from
// two forward passes and no stored walk:
//   pass 1 carries the tangent d/dE_in through each segment (Heun steps of
//     :444-551), giving a_k = dE_out/dE_in and c_k = d log g_k/dE_in (g_k the
//     segment's weight factor) and the V, H increments' partials; with the
//     prefix products P_k = a_1..a_k and sums C_k = sum_j c_j P_(j-1) the
//     energy adjoint of segment k is lambda_k = (A - C_k) / P_k, where
//     A = lambda_N P_N + C_N is known at the end of the path;
//   pass 2 carries d/dE_in and d/dw_k through the cell segments, forms
//     d log f / d w_k = lambda_k b_k + d_k (+ the V, H terms), and the warp
//     sums the samples' contributions per segment in a fixed order.
// This is the exact derivative of the discrete walk, the quantity the
// reference's segment rules (src/Tomography_rules.jl:33-106) chain with Zygote.
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace dp {
namespace wt {

constexpr double kMaxGain = 0.02;  // CSDA_MAX_RELATIVE_GAIN (src/Tomography.jl:89)
constexpr double kMaxStep = 60.0;  // CSDA_MAX_STEP_M (src/Tomography.jl:90)
constexpr int kMaxChunks = 8;      // energy samples per direction <= 32 * kMaxChunks
constexpr int kThreads = 128;

// Staged column slots: energies, log energies, then per material
// (rock, water, porous) CSDA and restricted stopping power and straggling,
// then the air's CSDA stopping power.
enum Slot { S_E = 0, S_LE, R_CS, R_MS, R_ST, W_CS, W_MS, W_ST, P_CS, P_MS, P_ST, A_CS, kSlots };

struct Params {
  TabView tv;                  // FP64 tables in global memory (grid layout)
  const double* col[kSlots];   // the staged columns (global addresses)
  uint32_t col_bytes;
  int porous;                  // porous material present
  double rho_rock, rho_water, rho_porous, porous_top;
  double det_elev, primary, mass, ctau;
  int corr;
  double ks, kh, ra, rb, rc, rd;
  int mcorr;
  double lin, quad;
  long n_bins;
  const double *cos_t, *rem, *exit_z;
  const int32_t* valid;
  const int64_t* seg_ptr;
  const int32_t* seg_cell;
  const double* seg_len;
  const uint8_t* shallow;
  const double* wf;
  long n_cells;
  int n_e;
  const double *E, *q, *ew;
  double* flux;
  double* jac;
  int* err_flag;
  unsigned long long* next_bin;  // bins handed out so far (zeroed before the launch)
  int wait_iters;                // polls of the table-staging wait
};

// Per-sample results of pass 1.
struct Lane {
  double f;       // w * corr * flux_gccly of the sample (0 when the walk is invalid)
  double A;       // lambda_N P_N + C_N (+ alpha terms)
  double aV, aH;  // d log corr / dV, d log corr / dH
};

__device__ __forceinline__ bool cell_porous(const Params& P, int cell) {
  return P.porous && P.porous_top > 0.0 && P.shallow && P.shallow[cell];
}
// cell_density (src/Tomography.jl:303-310) in FP64 and its derivative in w.
__device__ __forceinline__ double density64(const Params& P, int cell, double* dw = nullptr) {
  const double w = P.wf[cell];
  double s, ds;
  if (cell_porous(P, cell)) {
    s = 0.5 * (1.0 - w) / P.rho_porous + 0.5 * (1.0 - w) / P.rho_rock + w / P.rho_water;
    ds = -0.5 / P.rho_porous - 0.5 / P.rho_rock + 1.0 / P.rho_water;
  } else {
    s = (1.0 - w) / P.rho_rock + w / P.rho_water;
    ds = -1.0 / P.rho_rock + 1.0 / P.rho_water;
  }
  if (dw) *dw = -ds / (s * s);
  return 1.0 / s;
}

// Local spectral index b(E) of flux_gccly (src/Tomography.jl:367-372) and db/dE.
__device__ __forceinline__ void spectral_index(double E, double cs, double cs129, double* b,
                                               double* db) {
  const double eta = 1e-2;
  double dp, dm;
  double fp = gccly_flux(cs, cs129, E * (1.0 + eta), 1.0, &dp);
  double fm = gccly_flux(cs, cs129, E * (1.0 - eta), 1.0, &dm);
  *b = -(log(fp) - log(fm)) / (2 * eta);
  *db = -((1.0 + eta) * dp - (1.0 - eta) * dm) / (2 * eta);
}

// Deterministic warp sum (fixed shuffle tree).
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

}  // namespace wt
}  // namespace dp

#define WT_NS wt64
#define WT_REAL double
#include "wtomo_walk.cuh"
#undef WT_NS
#undef WT_REAL
#define WT_NS wt32
#define WT_REAL float
#include "wtomo_walk.cuh"
#undef WT_NS
#undef WT_REAL

namespace {

using namespace dp;

int check_config(dp_ctx* ctx, const dp_physics* ph, const dp_csda_config* c) {
  if (!c) return fail(ctx, DP_ERR_ARG, "null config");
  auto ok = [&](int m) { return m >= 0 && m < ph->n_mat; };
  if (!ok(c->rock_material) || !ok(c->water_material) || !ok(c->air_material) ||
      (c->porous_material >= 0 && !ok(c->porous_material)))
    return fail(ctx, DP_ERR_ARG, "material index outside the physics tables");
  if (!(c->rock_density > 0.0) || !(c->water_density > 0.0))
    return fail(ctx, DP_ERR_ARG, "positive rock and water densities required");
  if (c->porous_material >= 0 && c->porous_top_thickness > 0.0 && !(c->porous_density > 0.0))
    return fail(ctx, DP_ERR_ARG, "positive porous density required");
  return DP_OK;
}

// Enqueues the kernel on device arrays.
int run(dp_ctx* ctx, const dp_physics* ph, const dp_csda_config* c, const dp_csda_batch* B,
        long n_cells, const uint8_t* shallow, const double* wf, double* flux, double* jac,
        int precision) {
  int rc = check_config(ctx, ph, c);
  if (rc) return rc;
  if (B->n_energy < 1 || B->n_energy > 32 * wt::kMaxChunks)
    return fail(ctx, DP_ERR_ARG, "1 to 256 energy samples per call");
  wt::Params P{};
  P.tv = ph->view;
  const TabView& v = ph->view;
  const int porous = c->porous_material >= 0 ? c->porous_material : c->rock_material;
  const double* cols[wt::kSlots] = {
      v.col(c->rock_material, DP_COL_E),        v.col(c->rock_material, DP_COL_LOGE),
      v.col(c->rock_material, DP_COL_CSDA_S),   v.col(c->rock_material, DP_COL_MIXED_S),
      v.col(c->rock_material, DP_COL_STRAG),    v.col(c->water_material, DP_COL_CSDA_S),
      v.col(c->water_material, DP_COL_MIXED_S), v.col(c->water_material, DP_COL_STRAG),
      v.col(porous, DP_COL_CSDA_S),             v.col(porous, DP_COL_MIXED_S),
      v.col(porous, DP_COL_STRAG),              v.col(c->air_material, DP_COL_CSDA_S)};
  for (int s = 0; s < wt::kSlots; ++s) P.col[s] = cols[s];
  P.col_bytes = uint32_t(v.ld * sizeof(double));
  P.porous = c->porous_material >= 0 ? 1 : 0;
  P.rho_rock = c->rock_density;
  P.rho_water = c->water_density;
  P.rho_porous = c->porous_density;
  P.porous_top = c->porous_top_thickness;
  P.det_elev = c->detector_elevation;
  P.primary = c->primary_altitude;
  P.mass = ph->settings.mass;
  P.ctau = ph->settings.ctau;
  P.corr = c->correction;
  P.ks = c->kappa_strag;
  P.kh = c->kappa_hard;
  P.ra = c->resid_a;
  P.rb = c->resid_b;
  P.rc = c->resid_c;
  P.rd = c->resid_d;
  P.mcorr = c->material_correction;
  P.lin = c->material_linear;
  P.quad = c->material_quadratic;
  P.n_bins = B->n_bins;
  P.cos_t = B->cos_theta;
  P.rem = B->remaining_rock;
  P.exit_z = B->surface_exit_z;
  P.valid = B->valid;
  P.seg_ptr = B->seg_ptr;
  P.seg_cell = B->seg_cell;
  P.seg_len = B->seg_length;
  P.shallow = shallow;
  P.wf = wf;
  P.n_cells = n_cells;
  P.n_e = B->n_energy;
  P.E = B->energy;
  P.q = B->charge;
  P.ew = B->weight;
  P.flux = flux;
  P.jac = jac;
  P.err_flag = ctx->d_flag;
  P.next_bin = ctx->d_work;
  P.wait_iters = stage_wait(ctx);
  if (precision != DP_PREC_FP64 && precision != DP_PREC_MIXED)
    return fail(ctx, DP_ERR_ARG, "precision must be DP_PREC_FP64 or DP_PREC_MIXED");
  const bool mixed = precision == DP_PREC_MIXED;
  // FP64 columns staged, plus their FP32 copy for the mixed instance
  const size_t smem = 16 + size_t(wt::kSlots) * P.col_bytes * (mixed ? 3 : 2) / 2;
  auto kernel = mixed ? wt32::wtomo_kernel : wt64::wtomo_kernel;
  DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          int(smem)));
  int per_sm = 0, n_sm = 0;
  DP_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, wt::kThreads,
                                                                   smem));
  DP_CHECK_CUDA(ctx, cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
  const long need = (B->n_bins + wt::kThreads / 32 - 1) / (wt::kThreads / 32);
  const long blocks = std::max(1L, std::min(need, long(std::max(per_sm, 1)) * n_sm));
  DP_CHECK_CUDA(ctx, cudaMemsetAsync(P.next_bin, 0, sizeof(unsigned long long), ctx->stream));
  timed_begin(ctx);
  kernel<<<int(blocks), wt::kThreads, smem, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, mixed ? (jac ? "dir_csda32_grad" : "dir_csda32") : (jac ? "dir_csda_grad" : "dir_csda"));
  return DP_OK;
}

int read_flag(dp_ctx* ctx) {
  int flag = 0;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
    if (flag == 3) return fail(ctx, DP_ERR_ARG, "segment cell outside the water-fraction vector");
    return fail(ctx, DP_ERR_STATE, "a table-staging wait exceeded its limit");
  }
  return DP_OK;
}

}  // namespace

extern "C" {

int dp_dir_csda_dev(dp_ctx* ctx, const dp_physics* ph, const dp_csda_config* cfg,
                    const dp_csda_batch* batch, long n_cells, const uint8_t* shallow,
                    const double* water_fraction, double* flux, double* jac, int precision) {
  if (!ctx || !ph || !batch || !water_fraction || !flux || batch->n_bins < 0 || n_cells < 0)
    return fail(ctx, DP_ERR_ARG, "bad arguments");
  if (batch->n_bins == 0) return DP_OK;
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  int rc = run(ctx, ph, cfg, batch, n_cells, shallow, water_fraction, flux, jac, precision);
  if (rc) return rc;
  return ctx->blocking ? read_flag(ctx) : DP_OK;
}

int dp_dir_csda(dp_ctx* ctx, const dp_physics* ph, const dp_csda_config* cfg,
                const dp_csda_batch* B, long n_cells, const uint8_t* shallow,
                const double* water_fraction, double* flux, double* jac, int precision) {
  if (!ctx || !ph || !B || !water_fraction || !flux || B->n_bins < 0 || n_cells < 0)
    return fail(ctx, DP_ERR_ARG, "bad arguments");
  const long nb = B->n_bins;
  if (nb == 0) return DP_OK;
  if (!B->cos_theta || !B->remaining_rock || !B->surface_exit_z || !B->seg_ptr || !B->energy ||
      !B->charge || !B->weight)
    return fail(ctx, DP_ERR_ARG, "bad batch arrays");
  if (B->seg_ptr[0] != 0) return fail(ctx, DP_ERR_ARG, "segment offsets must start at 0");
  for (long b = 0; b < nb; ++b)
    if (B->seg_ptr[b + 1] < B->seg_ptr[b]) return fail(ctx, DP_ERR_ARG, "offsets must not decrease");
  const long ns = long(B->seg_ptr[nb]);
  for (long k = 0; k < ns; ++k) {
    if (B->seg_cell[k] < 0 || B->seg_cell[k] >= n_cells)
      return fail(ctx, DP_ERR_ARG, "segment cell outside the water-fraction vector");
    if (!(B->seg_length[k] >= 0.0)) return fail(ctx, DP_ERR_ARG, "nonnegative segment lengths required");
  }
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t db = size_t(nb) * 8, ne = size_t(B->n_energy) * 8;
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, 3 * db + 2 * (db + 8) + size_t(nb) * 4 + size_t(ns) * 28 +
                                               size_t(n_cells) * 9 + 3 * ne + 20 * 256, 2));
  A.cap = ctx->slot_bytes[2];
  double* ct = A.take<double>(nb);
  double* rr = A.take<double>(nb);
  double* ez = A.take<double>(nb);
  int32_t* va = B->valid ? A.take<int32_t>(nb) : nullptr;
  int64_t* sp = A.take<int64_t>(nb + 1);
  int32_t* sc = A.take<int32_t>(ns);
  double* sl = A.take<double>(ns);
  uint8_t* sh = shallow ? A.take<uint8_t>(n_cells) : nullptr;
  double* w = A.take<double>(n_cells);
  double* dE = A.take<double>(B->n_energy);
  double* dq = A.take<double>(B->n_energy);
  double* dw = A.take<double>(B->n_energy);
  double* fl = A.take<double>(nb);
  double* jc = jac ? A.take<double>(ns) : nullptr;
  if (!fl || (jac && !jc)) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  cudaStream_t s = ctx->stream;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return bytes && dst ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
  };
  cudaError_t e = cudaSuccess;
  for (auto r : {up(ct, B->cos_theta, db), up(rr, B->remaining_rock, db),
                 up(ez, B->surface_exit_z, db), up(va, B->valid, size_t(nb) * 4),
                 up(sp, B->seg_ptr, db + 8), up(sc, B->seg_cell, size_t(ns) * 4),
                 up(sl, B->seg_length, size_t(ns) * 8), up(sh, shallow, size_t(n_cells)),
                 up(w, water_fraction, size_t(n_cells) * 8), up(dE, B->energy, ne),
                 up(dq, B->charge, ne), up(dw, B->weight, ne)})
    if (r != cudaSuccess) e = r;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpyAsync");
  dp_csda_batch D = *B;
  D.cos_theta = ct;
  D.remaining_rock = rr;
  D.surface_exit_z = ez;
  D.valid = va;
  D.seg_ptr = sp;
  D.seg_cell = sc;
  D.seg_length = sl;
  D.energy = dE;
  D.charge = dq;
  D.weight = dw;
  int rc = run(ctx, ph, cfg, &D, n_cells, sh, w, fl, jc, precision);
  if (rc) return rc;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(flux, fl, db, cudaMemcpyDeviceToHost, s));
  if (jac && ns) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(jac, jc, size_t(ns) * 8, cudaMemcpyDeviceToHost, s));
  return read_flag(ctx);
}

}  // extern "C"

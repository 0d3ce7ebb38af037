// internal.h -- host-side definitions shared by the libdpgpu translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "common.cuh"

struct dp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;      // stream every launch of this context uses
  cudaStream_t own_stream = nullptr;  // created by dp_init
  // Launch accounting and optional per-kernel timing (CUDA events on `stream`).
  long long launches = 0;
  int timing = 0;
  // 1: every device-pointer call synchronises and checks the kernels' error
  // flag before returning; 0: calls return after enqueueing, dp_sync checks.
  int blocking = 1;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  struct Pending {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;        // recorded, not yet resolved (no host sync)
  std::vector<cudaEvent_t> spare;      // recycled events
  struct KTime {
    std::string name;
    double ms;
    long long n;  // timed launches
  };
  std::vector<KTime> ktime;
  std::string err;
  // Grow-only device scratch slots, reused across calls on this context.
  void* slot[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t slot_bytes[4] = {0, 0, 0, 0};
  int* d_flag = nullptr;  // device error flag (bounded waits that gave up)
  unsigned long long* d_work = nullptr;  // work counter of dynamically scheduled kernels
  // CTA size of the persistent transport kernels per family (DP_KERNEL_MC,
  // DP_KERNEL_DIR) and precision (DP_PREC_FP64, DP_PREC_MIXED); 0: default.
  int mc_threads[2][2] = {{0, 0}, {0, 0}};
  // Table staging (0: media in shared memory when they fit, 1: read through
  // L1/L2) of the same kernels; mixed precision reads them through L1/L2 by
  // default (its kernels leave the SM's shared memory to the L1 cache).
  int mc_stage[2][2] = {{0, 1}, {0, 1}};
  // Hand-out order of the histories (0: longest first, 1: index order).
  int mc_order[2][2] = {{0, 0}, {0, 0}};
  // CTA-lockstep phases (bit k: phase k), mixed precision only: both phases
  // of the two-layer transport and the mixed phase of the fixed-path one by
  // default.
  int mc_sync[2][2] = {{0, 3}, {0, 2}};
  // Energy nodes of the last host-pointer tomography evaluation (energies,
  // charges, weights) and their device copy: a call with the same nodes
  // uploads none.
  std::vector<double> nodes_host;
  double* nodes_dev = nullptr;
  // Limits lowered for failure-path tests (dp_set_debug_limits); negative:
  // the default (2,000,000 transport steps, 100,000 hard events per mixed
  // step, dp::kStageWait polls of a table-staging wait).
  int dbg_step_cap = -1, dbg_event_cap = -1, dbg_wait = -1;
};

namespace dp {
constexpr int kStepCap = 2000000;  // transport steps of one history
constexpr int kEventCap = 100000;  // hard events of one mixed step (src/MixedTransport.jl:157)
inline int step_cap(const dp_ctx* c) { return c->dbg_step_cap >= 0 ? c->dbg_step_cap : kStepCap; }
inline int event_cap(const dp_ctx* c) { return c->dbg_event_cap >= 0 ? c->dbg_event_cap : kEventCap; }
inline int stage_wait(const dp_ctx* c) { return c->dbg_wait >= 0 ? c->dbg_wait : kStageWait; }
struct HostElement {
  double Z, A, I, fraction;
};
struct HostMaterial {
  std::string name;
  double density = 0, I = 0, ZoA = 0;
  std::vector<HostElement> elements;
};
void build_empirical_table(const HostMaterial& m, const dp_settings& st, int n, double Kmin,
                           double Kmax, double* cols);
// A PUMAS dE/dx table (src/DEDXLoader.jl:26-43) in GeV and kg/m^2.
struct DedxTable {
  double ZoA = 0;
  std::vector<double> K, ion, brems, pair, photo, S, R;
};
// load_dedx_file (src/DEDXLoader.jl:49-190); false with *err set on failure.
bool load_dedx_table(const char* path, DedxTable* t, std::string* err);
// create_material_table_from_dedx (src/Physics.jl:146-273): DP_NCOL x n
// columns on the file's grid (n = t.K.size()).
void build_dedx_table(const HostMaterial& m, const DedxTable& t, const dp_settings& st,
                      double* cols);
double host_dcs_moment(int proc, double Z, double A, double I, double mass, double K, double xlo,
                       double xhi, int mode);
// Brackets one named kernel launch with events when timing is enabled; the
// elapsed time is added to ctx->ktime[name] by timed_end (which waits for
// the second event).
void timed_begin(dp_ctx* ctx);
void timed_end(dp_ctx* ctx, const char* name);
// Sets ctx->err and returns code.
int fail(dp_ctx* ctx, int code, const std::string& msg);
int cuda_fail(dp_ctx* ctx, cudaError_t e, const char* where);
// Ensures scratch slot `slot` (0..3) holds at least `bytes`; returns nullptr
// on failure.  Slot contents do not survive a grow.  Slot use: 0 per-call
// temporaries of the MC and plain kernels, 1 Jacobian values of an
// evaluation, 2 device copies of host inputs, 3 one-shot ray paths.
void* scratch(dp_ctx* ctx, size_t bytes, int slot = 0);
// Stochastic run_backward_mc on single-material rock and air media (one line
// of sight, FP64 or mixed precision per p->precision); fills flux, sigma and
// the flagged-history count of *res.  Returns DP_ERR_DOMAIN / DP_ERR_STATE
// (with the results filled) where the reference would throw.
int mc_backward_stochastic(dp_ctx* ctx, const dp_physics* ph, const dp_mc_params* p, int rock,
                           int air, double threshold, dp_los_result* res);
// CSDA histories (tangent mode) of lines of sight: history i of the running
// offsets off[] takes its record's geometry and draws (seed, i).
// precision DP_PREC_MIXED: FP32 transport and tangent, FP64 positions.
int csda_los(dp_ctx* ctx, const dp_physics* ph, int rock, int air, double threshold, double low,
             uint64_t seed, const dp_los* los, const int64_t* off, long n_los, long n,
             double* contrib, double* dcontrib, int precision);
// Tomography internals used by the inversion loops (tomo.cu): evaluation into
// a caller-owned Jacobian buffer and J^T v on the resident paths' buckets.
int tomo_eval_raw(dp_ctx* ctx, const dp_physics* ph, const dp_paths* pa, const dp_tomo_params* tp,
                  const double* rho, double* flux, void* jraw, int precision);
// The bucketed Jacobian values in CSC order (nnz entries of out), for
// repeated J^T v products with csc = true.
int tomo_csc_values(dp_ctx* ctx, const dp_paths* pa, const void* jbuf, int precision, void* out);
int tomo_transpose(dp_ctx* ctx, const dp_paths* pa, const void* jbuf, int precision,
                   const double* cot, double* grad, bool csc = false);
// Bump allocator over one scratch slot (256-byte aligned pieces).
struct Arena {
  char* base = nullptr;
  size_t off = 0, cap = 0;
  template <class T>
  T* take(size_t n) {
    size_t a = (off + 255) & ~size_t(255);
    size_t b = a + (n ? n : 1) * sizeof(T);
    if (!base || b > cap) return nullptr;
    off = b;
    return reinterpret_cast<T*>(base + a);
  }
};
}  // namespace dp

struct dp_physics {
  dp_ctx* ctx = nullptr;
  int device = 0;  // the context's device (the free path must not read a destroyed context)
  dp_settings settings{};
  int n_mat = 0, n = 0, ld = 0;
  std::vector<double> host;           // n_mat x DP_NCOL x n
  std::vector<dp::HostMaterial> recipes;
  bool has_recipes = false;
  double* dev = nullptr;              // n_mat x DP_NCOL x ld
  dp::TabView view{};
  // Single-precision derived columns for the mixed-precision kernels:
  // n_mat x dp::kNC32 x ld32 floats (see dp::Col32).
  float* dev32 = nullptr;
  int ld32 = 0;
};

// Ray paths through a voxel grid, traced once (geometry does not depend on
// the densities): CSR segment lists plus the CSC permutation used by the
// deterministic J^T r gather.
struct dp_paths {
  dp_ctx* ctx = nullptr;
  int device = 0;  // the context's device (the free path must not read a destroyed context)
  dp_grid grid{};
  int side_cell = -1;
  long n_rays = 0;
  int64_t nnz = 0;      // segments, side-exit remainders included
  int max_seg = 0;      // longest segment list
  dp_ray* rays = nullptr;
  int64_t* row_ptr = nullptr;   // n_rays + 1
  int32_t* cell = nullptr;      // nnz (-1: side remainder at a fixed density)
  double* len = nullptr;        // nnz
  int32_t* row_of = nullptr;    // nnz
  int64_t* cptr = nullptr;      // ncell + 1
  int32_t* perm = nullptr;      // entries sorted by (cell, entry index)
  float4* geom = nullptr;       // per ray: cos_theta_star, its 1.29 power,
                                // 1/max(|cos theta|, 0.01), cos theta
  int32_t* order = nullptr;     // rays by decreasing segment count (schedule)
  int32_t* prow = nullptr;      // row_of[perm[p]] (gather reads it in order)
  int32_t* big = nullptr;       // cells whose bucket holds more than 32 entries
  int n_big = 0;
  bool owned = true;            // arrays allocated with cudaMalloc (else arena)
};

#define DP_CHECK_CUDA(ctx, call)                                  \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return dp::cuda_fail((ctx), e_, #call); \
  } while (0)

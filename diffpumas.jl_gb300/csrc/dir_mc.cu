// dir_mc.cu -- fixed-path backward Monte Carlo of libdpgpu
// (compute_directional_flux_mc, src/Tomography.jl:826-1041): many directions
// in one launch, each a list of cell segments (medium, density, length), the
// rock beyond the cells and the air above the surface.  Straggled steps
// below the mode switch, mixed steps above it, no scattering.  The history
// loop, the media packing and the tallies are shared with run_backward_mc
// (mc_loop.cuh, mc.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mc_host.h"
#include "mc_loop.cuh"

using namespace dp;
using namespace dp::mc;

// A media set of fixed-path runs with its device copies per precision.
struct dp_dir_media {
  dp_ctx* ctx = nullptr;
  const dp_physics* phys = nullptr;
  std::vector<const dp_mixture*> media;
  struct Dev {
    int precision = -1;
    unsigned char* blob = nullptr;  // n_media packed media
    MedInfo* info = nullptr;        // n_media
    Layout lay{};
    int nel = 0;
  };
  Dev dev[2];
};

namespace dp {
namespace mc {

constexpr int kDirMaxMedia = 256;

struct DirParams {
  const unsigned char* blob;  // packed media (n_media x lay.med_bytes)
  Layout lay;
  const MedInfo* info;
  int n_media, n_staged;      // media [0, n_staged) are copied to shared memory
  Consts C;
  uint64_t seed, id0;
  long n, n_dirs;
  dp_dir_batch B;             // device arrays
  double* contrib;
  int32_t* status;
  int32_t* steps;
  double* efinal;             // 2 per history: final energy, weight
  unsigned long long* counter;
  int* err_flag;
  int coop_nel, coop_stride, coop_kmax;  // batched DCS buffers: elements, floats per warp, events
  int coop_kc;  // events per chunk of the CTA buffer (lockstep phases)
  int sync;     // bit k: phase k runs its steps in CTA lockstep
  void* queue;
  void* start;
  void* end;
};

// Start record: sample weight, final energy, charge, direction.
template <class R>
struct DirStart {
  double ws;
  R E;
  float q;
  int dir;
};
template <class R>
struct DirEnd {
  R E, w;
  int status, steps;
};

// History state: the State plus its place on the path.  stage 0: cell
// segments, 1: rock beyond the cells, 2: air, 3: ended.
template <class R>
struct DirHist {
  State<R> s;
  Alt<R> dist;    // path length travelled (src/Geometry.jl State.distance)
  Alt<R> d0;      // path length before the step in flight
  R E0, limit;    // energy before the step, the step's energy limit
  R remaining;    // metres left in the current segment
  R rho, cos_t;   // segment density, cos(zenith) of the direction
  int seg, seg_end, stage, med, dir, steps;
  Cont<R> x;
};
template <class R>
struct DirHandoff {
  Alt<R> z, dist;
  R E, w, remaining, rho, cos_t;
  int status, steps, seg, seg_end, stage, med, dir, used;
  uint32_t block, w0, w1, w2, w3;
  long index;
  uint64_t stream;
};

// Path length since d0.
__device__ __forceinline__ double alt_since(double d, double d0) { return d - d0; }
__device__ __forceinline__ float alt_since(F2 d, F2 d0) { return alt_sub(d, d0); }
// Altitude in the transport precision.
__device__ __forceinline__ double alt_r(double z) { return z; }
__device__ __forceinline__ float alt_r(F2 z) { return z.h + z.l; }

// sample_energy_set (src/Tomography.jl:236-248) on the history's Philox block
// 0: log-uniform final energy with weight k rk, charge +-1 with p = 1/2.
__device__ __forceinline__ void dir_sample(uint64_t seed, uint64_t id, double emin, double emax,
                                           double* E, double* q, double* w) {
  U4 b = philox(U4{uint32_t(id), uint32_t(id >> 32), 0u, 0u}, uint32_t(seed), uint32_t(seed >> 32));
  if (!(emax > emin)) {
    *E = emin;
    *w = 1.0;
  } else {
    double rk = log(emax / emin);
    *E = emin * exp(rk * u01(b.x, b.y));
    *w = *E * rk;
  }
  *q = u01(b.z, b.w) > 0.5 ? 1.0 : -1.0;
}

// Direction of history i: dir with smp[dir] <= i < smp[dir + 1].
__device__ __forceinline__ int dir_of(const int64_t* smp, long n_dirs, long i) {
  long lo = 0, hi = n_dirs;
  while (hi - lo > 1) {
    long mid = (lo + hi) >> 1;
    if (smp[mid] <= i) lo = mid; else hi = mid;
  }
  return int(lo);
}

template <class R>
__global__ void __launch_bounds__(256) dir_init_kernel(const __grid_constant__ DirParams P) {
  DirStart<R>* out = static_cast<DirStart<R>*>(P.start);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < P.n;
       i += long(gridDim.x) * blockDim.x) {
    double E, q, w;
    if (P.B.energy) {
      E = P.B.energy[i];
      q = P.B.charge[i];
      w = P.B.weight[i];
    } else {
      dir_sample(P.seed, P.id0 + uint64_t(i), P.B.energy_min, P.B.energy_max, &E, &q, &w);
    }
    out[i] = DirStart<R>{w, R(E), float(q), dir_of(P.B.sample_ptr, P.n_dirs, i)};
  }
}

// Fixed-path geometry for the shared history loop (src/Tomography.jl:876-969).
template <class R>
struct PathGeo {
  using Hist = DirHist<R>;
  using Queue = DirHandoff<R>;
  const DirParams& P;
  const Med<R>* meds;
  __device__ long n0() const { return P.n; }
  __device__ const Med<R>& medium(int k) const { return meds[k]; }
  __device__ const Med<R>* media() const { return meds; }

  __device__ R thr() const { return sizeof(R) == 8 ? R(P.C.thr) : R(P.C.thr_f); }

  // Moves to the next segment with more than 1e-8 m to go (the reference's
  // loop conditions), or ends the path.
  __device__ void next_segment(Hist& h) const {
    for (;;) {
      if (h.stage == 0) {
        if (++h.seg < h.seg_end) {
          h.med = P.B.seg_medium[h.seg];
          h.rho = R(P.B.seg_density[h.seg]);
          h.remaining = R(P.B.seg_length[h.seg]);
        } else {
          h.stage = 1;
          h.med = P.B.rock_medium;
          h.rho = R(P.B.rock_density);
          h.remaining = R(P.B.remaining_rock[h.dir]);
        }
      } else if (h.stage == 1) {
        h.stage = 2;
        h.med = P.B.air_medium;
        h.rho = R(0);
        h.remaining = R(P.B.air_distance[h.dir]);
      } else {
        h.stage = 3;
        return;
      }
      if (h.med < 0 || h.med >= P.n_media) {  // device-array calls are not checked on the host
        h.s.status |= ST_BAD_MEDIUM;
        h.stage = 3;
        return;
      }
      if (h.remaining > R(1e-8)) return;
    }
  }

  __device__ void start(long i, Hist& h, Stream& g) const {
    const DirStart<R> r = static_cast<const DirStart<R>*>(P.start)[i];
    const int d = r.dir;
    h.dir = d;
    h.cos_t = R(P.B.cos_theta[d]);
    // initial_state (src/Tomography.jl:863-869): direction -dir
    h.s.z = alt_make<R>(0.0);
    h.dist = alt_make<R>(0.0);
    h.s.ux = R(0);
    h.s.uy = R(0);
    h.s.uz = -h.cos_t;
    h.s.E = r.E;
    h.s.w = R(1);
    h.s.status = 0;
    h.steps = 0;
    h.x.kind = CONT_NONE;
    h.seg = int(P.B.seg_ptr[d]) - 1;
    h.seg_end = int(P.B.seg_ptr[d + 1]);
    h.stage = 0;
    h.remaining = R(0);
    if (P.B.valid && !P.B.valid[d]) h.stage = 3;
    else next_segment(h);
    g.init(P.seed, P.id0 + uint64_t(i));
  }

  __device__ void save(const Hist& h, const Stream& g, long i, Queue* q) const {
    Queue v;
    v.z = h.s.z;
    v.dist = h.dist;
    v.E = h.s.E;
    v.w = h.s.w;
    v.remaining = h.remaining;
    v.rho = h.rho;
    v.cos_t = h.cos_t;
    v.status = h.s.status;
    v.steps = h.steps;
    v.seg = h.seg;
    v.seg_end = h.seg_end;
    v.stage = h.stage;
    v.med = h.med;
    v.dir = h.dir;
    v.used = g.used;
    v.block = g.block;
    v.w0 = g.w0;
    v.w1 = g.w1;
    v.w2 = g.w2;
    v.w3 = g.w3;
    v.index = i;
    v.stream = uint64_t(g.c0) | (uint64_t(g.c1) << 32);
    *q = v;
  }
  __device__ long load(const Queue& v, Hist& h, Stream& g) const {
    h.s.z = v.z;
    h.dist = v.dist;
    h.s.ux = R(0);
    h.s.uy = R(0);
    h.s.uz = -v.cos_t;
    h.s.E = v.E;
    h.s.w = v.w;
    h.s.status = v.status;
    h.remaining = v.remaining;
    h.rho = v.rho;
    h.cos_t = v.cos_t;
    h.steps = v.steps;
    h.seg = v.seg;
    h.seg_end = v.seg_end;
    h.stage = v.stage;
    h.med = v.med;
    h.dir = v.dir;
    h.x.kind = CONT_NONE;
    g.init(P.seed, v.stream);
    g.block = v.block;
    g.used = v.used;
    g.w0 = v.w0;
    g.w1 = v.w1;
    g.w2 = v.w2;
    g.w3 = v.w3;
    return v.index;
  }
  __device__ void end(long i, const Hist& h) const {
    static_cast<DirEnd<R>*>(P.end)[i] = DirEnd<R>{h.s.E, h.s.w, h.s.status, h.steps};
  }

  // Bookkeeping after a completed step of `moved` metres (src/Tomography.jl:904-917):
  // the reference's distance difference of its State.
  __device__ int step_end(Hist& h, R moved) const {
    State<R>& s = h.s;
    if (++h.steps > P.C.step_cap) s.status |= ST_STEP_CAP;
    if (s.status & ST_FATAL) return ADV_DONE;
    alt_add(h.dist, moved);
    const R actual = R(alt_since(h.dist, h.d0));
    if (!(s.w > R(0)) || !isfinite(s.w)) return ADV_DONE;
    const R top = thr();
    // a sub-ulp displacement that reached the mode boundary is progress
    if (actual <= R(0) && h.E0 < h.limit && h.limit < top && s.E >= h.limit) return ADV_STEP;
    if (!(actual > R(0))) {
      if (!(s.E >= top)) s.status |= ST_NO_PROGRESS;
      return ADV_DONE;
    }
    h.remaining = fmax(R(0), h.remaining - actual);
    return ADV_STEP;
  }

  template <bool COOP, int PHASE>
  __device__ int advance(Hist& h, Stream& g) const {
    const Consts& C = P.C;
    const double eps = kEps64;
    State<R>& s = h.s;
    const R top = thr();
    const R low = sizeof(R) == 8 ? R(C.thr_low) : R(C.thr_low_f);
    for (;;) {
      if (h.stage == 3) return ADV_DONE;
      // at the energy limit every later segment is skipped and the history
      // contributes nothing (the source-energy cut)
      if (sizeof(R) == 8 ? !(double(s.E) < C.thr - eps) : !(s.E < top)) return ADV_DONE;
      if (!(h.remaining > R(1e-8))) {
        next_segment(h);
        continue;
      }
      break;
    }
    if (!(s.w > R(0)) || !isfinite(s.w)) return ADV_DONE;
    const bool below = sizeof(R) == 8 ? double(s.E) < C.thr_low - eps : s.E < low;
    if (PHASE == 0 && !below) return ADV_HANDOFF;
    if (PHASE == 1 && below) {  // not reached: the energy never decreases
      s.status |= ST_OUTER_CAP;
      return ADV_DONE;
    }
    const R limit = below ? fmin(low, top) : top;
    const Med<R>& m = meds[h.med];
    const bool air = h.stage == 2;
    // locals_air_at_altitude (src/Geometry.jl:95-106) at detector elevation + z
    const R rho = air ? R(1.205) * exp(-(R(P.B.detector_elevation) + alt_r(s.z)) / R(12e3)) : h.rho;
    const Loc<R> Li = locate(m, s.E);
    R mx = R(0.01) * at(m, Li, MC_CR) / fmax(rho, air ? R(1e-8) : R(1e-6));
    if (air) mx = fmin(mx, R(0.05 * 12e3) / fmax(h.cos_t, R(0.05)));
    const R step = fmin(h.remaining, fmax(R(1e-6), fmin(h.remaining + R(1e-7), mx)));
    h.d0 = h.dist;
    h.E0 = s.E;
    h.limit = limit;
    if (C.straggling) {
      if constexpr (PHASE == 0) {
        if (straggled_step<R, COOP, true, true>(m, C, s, Li, R(0), rho, step, g, false, limit,
                                                h.x)) {
          h.x.kind = CONT_STRAG;
          h.x.medium = h.med;
          return ADV_WAIT;
        }
        return step_end(h, h.x.moved);
      } else {
        if (mixed_step<R, COOP, true>(m, C, s, rho, step, g, limit, h.x)) {
          h.x.kind = CONT_MIXED;
          h.x.medium = h.med;
          return ADV_WAIT;
        }
        return step_end(h, mixed_moved(h.x));
      }
    }
    csda_step(m, C, s, Li, rho, step);
    return step_end(h, step);
  }

  template <int PHASE>
  __device__ int resume(Hist& h, Stream& g) const {
    Cont<R>& x = h.x;
    const Med<R>& m = meds[x.medium];
    x.kind = CONT_NONE;
    const DelOutT<R> d = del_end(x.anc, x.denom, x.total, x.pick);
    if constexpr (PHASE == 1) {
      const R Emax = m.kcol(K_E)[m.nk - 1];
      if (mixed_event(h.s, x, d)) {
        mixed_end(h.s, x, Emax, h.limit, false);
      } else {
        ++x.event;
        if (mixed_run_in<R, true>(m, P.C, h.s, x, g, h.limit)) {
          x.kind = CONT_MIXED;
          return ADV_WAIT;
        }
      }
      return step_end(h, mixed_moved(x));
    } else {
      Loc<R> Li = locate(m, x.r0);
      // the fixed-path transport never scatters (x.flag is 0)
      const R moved = straggled_end_in(m, P.C, h.s, Li, R(0), x.r0, d.energy, x.r1, x.r2, d.weight,
                                       d.process, d.element, true, false, R(0), x.r3, x.a, true,
                                       false, g);
      return step_end(h, moved);
    }
  }
};

// Shared memory: [0,16) mbarrier, staged media, the media descriptors, the
// warps' DCS buffers.
template <class R>
__host__ __device__ inline uint32_t dir_desc_offset(const DirParams& P) {
  return 16u + uint32_t(P.n_staged) * P.lay.med_bytes;
}
template <class R>
__host__ __device__ inline uint32_t dir_coop_offset(const DirParams& P) {
  return dir_desc_offset<R>(P) + (uint32_t(P.n_media * sizeof(Med<R>)) + 15u) / 16u * 16u;
}

template <class R, int PHASE, int T>
__global__ void __launch_bounds__(T, 1) dir_kernel(const __grid_constant__ DirParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t tables = uint32_t(P.n_staged) * P.lay.med_bytes;
  if (tables && !stage_blob(smem + 16, P.blob, tables, reinterpret_cast<uint64_t*>(smem),
                            P.C.wait_iters)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    PathGeo<R> geo{P, nullptr};
    drain_histories<R, PHASE>(geo, P.counter, static_cast<DirHandoff<R>*>(P.queue));
    return;
  }
  Med<R>* meds = reinterpret_cast<Med<R>*>(smem + dir_desc_offset<R>(P));
  for (int k = threadIdx.x; k < P.n_media; k += blockDim.x) {
    const unsigned char* b =
        k < P.n_staged ? smem + 16 + size_t(k) * P.lay.med_bytes : P.blob + size_t(k) * P.lay.med_bytes;
    meds[k] = make_med<R>(b, P.lay, P.info[k]);
  }
  __syncthreads();
  PathGeo<R> geo{P, meds};
  float* coop = reinterpret_cast<float*>(smem + dir_coop_offset<R>(P));
  transport_histories<R, PHASE, KCfg<R>::coop>(geo, P.C, P.counter,
                                               static_cast<DirHandoff<R>*>(P.queue), coop,
                                               P.coop_stride, P.coop_kmax, P.coop_kc, P.coop_nel,
                                               nullptr, ((P.sync >> PHASE) & 1) != 0);
}

// Contribution 2 w_i w flux_gccly(cos zenith, E, q) of every ended history
// (src/Tomography.jl:1027-1033), FP64.
template <class R>
__global__ void __launch_bounds__(256) dir_finish_kernel(const __grid_constant__ DirParams P) {
  const DirStart<R>* st = static_cast<const DirStart<R>*>(P.start);
  const DirEnd<R>* en = static_cast<const DirEnd<R>*>(P.end);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < P.n;
       i += long(gridDim.x) * blockDim.x) {
    const DirEnd<R> e = en[i];
    const DirStart<R> r = st[i];
    double c = 0.0;
    const bool valid = !P.B.valid || P.B.valid[r.dir];
    if (valid && !(e.status & ST_FATAL) && e.w > R(0) && isfinite(e.w) && double(e.E) < P.C.thr) {
      double cs = cos_theta_star(P.B.cos_theta[r.dir]);
      c = 2.0 * r.ws * double(e.w) * gccly_flux(cs, pow(cs, 1.29), double(e.E), double(r.q), nullptr);
    }
    P.contrib[i] = c;
    P.status[i] = e.status;
    if (P.steps) P.steps[i] = e.steps;
    if (P.efinal) {
      P.efinal[2 * i] = double(e.E);
      P.efinal[2 * i + 1] = double(e.w);
    }
  }
}

}  // namespace mc
}  // namespace dp

namespace {

constexpr size_t kDirRecBytes =
    sizeof(DirHandoff<double>) + sizeof(DirStart<double>) + sizeof(DirEnd<double>) + 64;

int dir_device(dp_ctx* ctx, dp_dir_media* M, int precision, dp_dir_media::Dev** out) {
  dp_dir_media::Dev& D = M->dev[precision == DP_PREC_MIXED ? 1 : 0];
  if (D.blob) {
    *out = &D;
    return DP_OK;
  }
  const size_t es = precision == DP_PREC_MIXED ? sizeof(float) : sizeof(double);
  const int n = int(M->media.size());
  Layout L = make_layout(M->media.data(), n, es);
  std::vector<unsigned char> h(size_t(n) * L.med_bytes);
  std::vector<MedInfo> info(n);
  int nel = 0;
  for (int k = 0; k < n; ++k) {
    pack_medium(M->media[k], L, es, h.data() + size_t(k) * L.med_bytes);
    info[k] = make_info(M->media[k]);
    nel = std::max(nel, M->media[k]->nel);
  }
  DP_CHECK_CUDA(ctx, cudaMalloc(&D.blob, h.size()));
  DP_CHECK_CUDA(ctx, cudaMalloc(&D.info, sizeof(MedInfo) * n));
  DP_CHECK_CUDA(ctx, cudaMemcpy(D.blob, h.data(), h.size(), cudaMemcpyHostToDevice));
  DP_CHECK_CUDA(ctx, cudaMemcpy(D.info, info.data(), sizeof(MedInfo) * n, cudaMemcpyHostToDevice));
  D.precision = precision;
  D.lay = L;
  D.nel = nel;
  *out = &D;
  return DP_OK;
}

template <class R, int PHASE, int T>
int dir_phase(dp_ctx* ctx, const DirParams& P, size_t smem, long max_blocks) {
  const int threads = T;
  DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(dir_kernel<R, PHASE, T>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(dir_kernel<R, PHASE, T>,
                                          cudaFuncAttributePreferredSharedMemoryCarveout,
                                          carveout_percent(ctx->device, smem)));
  int per_sm = 0, n_sm = 0;
  DP_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dir_kernel<R, PHASE, T>,
                                                                   threads, smem));
  DP_CHECK_CUDA(ctx, cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
  if (per_sm < 1) return fail(ctx, DP_ERR_CUDA, "fixed-path MC kernel does not fit on a multiprocessor");
  long blocks = std::max(1L, std::min(long(per_sm) * n_sm, max_blocks));
  timed_begin(ctx);
  dir_kernel<R, PHASE, T><<<int(blocks), threads, smem, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, sizeof(R) == 4 ? (PHASE ? "dir_mixed_hi" : "dir_mixed_lo")
                                : (PHASE ? "dir_fp64_hi" : "dir_fp64_lo"));
  return DP_OK;
}

template <class R, int T>
int dir_launch_t(dp_ctx* ctx, DirParams& P) {
  const int threads = T;
  const int warps = threads / 32;
  P.coop_kmax = 1;
  P.coop_kc = 0;
  P.sync = ctx->mc_sync[DP_KERNEL_DIR][sizeof(R) == 4];
  P.coop_stride = KCfg<R>::coop ? coop_floats(P.coop_nel, 1) : 0;
  size_t coop_bytes = size_t(warps) * P.coop_stride * sizeof(float);
  int dev_smem = 0;
  DP_CHECK_CUDA(ctx, cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
  // stage the leading media that fit (none when the context reads the
  // tables through L1/L2)
  P.n_staged = 0;
  const bool stage = ctx->mc_stage[DP_KERNEL_DIR][sizeof(R) == 4] == 0;
  for (int k = stage ? P.n_media : 0; k >= 0; --k) {
    P.n_staged = k;
    if (dir_coop_offset<R>(P) + coop_bytes <= size_t(dev_smem)) break;
  }
  if (KCfg<R>::coop) {
    // the shared memory left after the staged media, up to the smallest
    // carve-out step that holds a one-event-per-warp buffer, batches DCS sums
    const size_t cap = std::min(size_t(dev_smem), carveout_cap(dir_coop_offset<R>(P) + coop_bytes));
    P.coop_kmax = coop_kmax(cap - std::min(cap, size_t(dir_coop_offset<R>(P))), warps, P.coop_nel);
    P.coop_stride = coop_floats(P.coop_nel, P.coop_kmax);
    coop_bytes = size_t(warps) * P.coop_stride * sizeof(float);
    P.coop_kc = cta_kc(warps * P.coop_stride, P.coop_nel, threads);
  }
  const size_t smem = dir_coop_offset<R>(P) + coop_bytes;
  if (smem > size_t(dev_smem)) return fail(ctx, DP_ERR_ARG, "too many media for the fixed-path MC kernel");
  const long need = (P.n + threads - 1) / threads;
  const long rec_blocks = std::min((P.n + 255) / 256, 152L * 32);
  DP_CHECK_CUDA(ctx, cudaMemsetAsync(P.counter, 0, 3 * sizeof(unsigned long long), ctx->stream));
  timed_begin(ctx);
  dir_init_kernel<R><<<int(rec_blocks), 256, 0, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "dir_init");
  int rc = dir_phase<R, 0, T>(ctx, P, smem, need);
  if (!rc) rc = dir_phase<R, 1, T>(ctx, P, smem, need);
  if (rc) return rc;
  timed_begin(ctx);
  dir_finish_kernel<R><<<int(rec_blocks), 256, 0, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "dir_finish");
  return DP_OK;
}

template <class R>
int dir_launch(dp_ctx* ctx, DirParams& P) {
  return with_threads<R>(ctx->mc_threads[DP_KERNEL_DIR][sizeof(R) == 4],
                         [&](auto t) { return dir_launch_t<R, decltype(t)::value>(ctx, P); });
}

// Enqueues one run over the batch (device arrays) and the per-direction
// tallies; *bits receives the device word of OR-ed history status bits.
int dir_run(dp_ctx* ctx, const dp_physics* ph, dp_dir_media* M, const dp_dir_batch* B,
            long total, const dp_mc_config* cfg, dp_los_result* d_out, int** bits_out,
            double** contrib_out, int32_t** status_out, double** final_out) {
  Consts C;
  int rc = check_cfg(ctx, ph, cfg, &C);
  if (rc) return rc;
  if (cfg->scattering)
    return fail(ctx, DP_ERR_ARG,
                "Fixed RayPath MC supports energy-loss fluctuations only; scattering requires geometry retracing");
  const int n_media = int(M->media.size());
  if (B->rock_medium < 0 || B->rock_medium >= n_media || B->air_medium < 0 ||
      B->air_medium >= n_media)
    return fail(ctx, DP_ERR_ARG, "rock_medium and air_medium must index the media set");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  dp_dir_media::Dev* D = nullptr;
  rc = dir_device(ctx, M, cfg->precision, &D);
  if (rc) return rc;
  const long nd = B->n_dirs, nt = total > 0 ? total : 1;
  Arena A;
  A.base = static_cast<char*>(scratch(
      ctx, size_t(nt) * (12 + 4 + 16 + kDirRecBytes) + size_t(nd + 1) * 16 +
               size_t(tally_jobs(nd, nt)) * tally_part_bytes() + 4096, 0));
  A.cap = ctx->slot_bytes[0];
  double* dc = A.take<double>(nt);
  int32_t* ds = A.take<int32_t>(nt);
  int64_t* off = A.take<int64_t>(nd + 1);
  int64_t* coff = A.take<int64_t>(nd + 1);
  unsigned char* tpart = A.take<unsigned char>(size_t(tally_jobs(nd, nt)) * tally_part_bytes());
  unsigned long long* ctr = A.take<unsigned long long>(3);
  DirHandoff<double>* queue = A.take<DirHandoff<double>>(nt);
  DirStart<double>* srec = A.take<DirStart<double>>(nt);
  DirEnd<double>* erec = A.take<DirEnd<double>>(nt);
  double* fin = final_out ? A.take<double>(2 * nt) : nullptr;
  int* bits = A.take<int>(1);
  if (!bits) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  DP_CHECK_CUDA(ctx, cudaMemsetAsync(bits, 0, sizeof(int), ctx->stream));
  rc = group_offsets(ctx, nullptr, B->sample_ptr, nd, off, coff, total);
  if (rc) return rc;
  if (total > 0) {
    DirParams P{};
    P.blob = D->blob;
    P.lay = D->lay;
    P.info = D->info;
    P.n_media = n_media;
    P.C = C;
    P.seed = cfg->seed;
    P.id0 = 0;
    P.n = total;
    P.n_dirs = nd;
    P.B = *B;
    P.contrib = dc;
    P.status = ds;
    P.efinal = fin;
    P.counter = ctr;
    P.err_flag = ctx->d_flag;
    P.coop_nel = D->nel;
    P.queue = queue;
    P.start = srec;
    P.end = erec;
    rc = cfg->precision == DP_PREC_MIXED ? dir_launch<float>(ctx, P) : dir_launch<double>(ctx, P);
    if (rc) return rc;
  }
  rc = group_tally(ctx, dc, ds, nullptr, nullptr, nullptr, B->valid, nd, total, 1, off, coff, tpart,
                   d_out, bits);
  if (rc) return rc;
  if (bits_out) *bits_out = bits;
  if (contrib_out) *contrib_out = dc;
  if (status_out) *status_out = ds;
  if (final_out) *final_out = fin;
  return DP_OK;
}

}  // namespace

extern "C" {

int dp_dir_media_create(dp_ctx* ctx, const dp_physics* ph, int n_media,
                        const dp_mixture* const* media, dp_dir_media** out) {
  if (!ctx || !ph || !media || !out) return fail(ctx, DP_ERR_ARG, "null argument");
  if (n_media < 1 || n_media > kDirMaxMedia)
    return fail(ctx, DP_ERR_ARG, "a media set holds 1 to 256 media");
  for (int k = 0; k < n_media; ++k) {
    if (!media[k]) return fail(ctx, DP_ERR_ARG, "null medium");
    if (media[k]->phys != ph || media[k]->n != media[0]->n || media[k]->nk != media[0]->nk)
      return fail(ctx, DP_ERR_ARG, "media must come from one physics");
  }
  dp_dir_media* M = new dp_dir_media;
  M->ctx = ctx;
  M->phys = ph;
  M->media.assign(media, media + n_media);
  *out = M;
  return DP_OK;
}

int dp_dir_media_free(dp_dir_media* M) {
  if (!M) return DP_OK;
  for (auto& D : M->dev) {
    cudaFree(D.blob);
    cudaFree(D.info);
  }
  cudaGetLastError();  // a failed release must not surface at a later launch
  delete M;
  return DP_OK;
}

int dp_dir_mc_dev(dp_ctx* ctx, const dp_physics* ph, dp_dir_media* M, const dp_dir_batch* B,
                  long total_samples, const dp_mc_config* cfg, dp_los_result* out) {
  if (!ctx || !ph || !M || !B || !out || B->n_dirs <= 0 || total_samples < 0)
    return fail(ctx, DP_ERR_ARG, "bad arguments");
  if (!B->cos_theta || !B->remaining_rock || !B->air_distance || !B->seg_ptr || !B->sample_ptr ||
      (!B->energy && !(B->energy_min > 0.0)) || (B->energy && (!B->charge || !B->weight)))
    return fail(ctx, DP_ERR_ARG, "bad batch arrays");
  int* bits = nullptr;
  int rc = dir_run(ctx, ph, M, B, total_samples, cfg, out, &bits, nullptr, nullptr, nullptr);
  if (rc) return rc;
  if (ctx->blocking) return status_result(ctx, bits);
  return DP_OK;
}

int dp_dir_mc(dp_ctx* ctx, const dp_physics* ph, dp_dir_media* M, const dp_dir_batch* B,
              const dp_mc_config* cfg, dp_los_result* out, double* contrib, int32_t* status,
              double* final_state) {
  if (!ctx || !ph || !M || !B || !out || B->n_dirs <= 0) return fail(ctx, DP_ERR_ARG, "bad arguments");
  const long nd = B->n_dirs;
  if (!B->cos_theta || !B->remaining_rock || !B->air_distance || !B->seg_ptr || !B->sample_ptr)
    return fail(ctx, DP_ERR_ARG, "bad batch arrays");
  if (B->seg_ptr[0] != 0 || B->sample_ptr[0] != 0) return fail(ctx, DP_ERR_ARG, "offsets must start at 0");
  for (long d = 0; d < nd; ++d)
    if (B->seg_ptr[d + 1] < B->seg_ptr[d] || B->sample_ptr[d + 1] < B->sample_ptr[d])
      return fail(ctx, DP_ERR_ARG, "offsets must not decrease");
  const long ns = long(B->seg_ptr[nd]), n = long(B->sample_ptr[nd]);
  if (ns > 2147483647L) return fail(ctx, DP_ERR_ARG, "at most 2^31 - 1 segments per batch");
  const int n_media = int(M->media.size());
  for (long j = 0; j < ns; ++j) {
    if (B->seg_medium[j] < 0 || B->seg_medium[j] >= n_media)
      return fail(ctx, DP_ERR_ARG, "segment medium outside the media set");
    // transport steps need a positive density (src/MixedTransport.jl:146)
    if (!(B->seg_density[j] > 0.0) || !(B->seg_length[j] >= 0.0))
      return fail(ctx, DP_ERR_ARG, "positive segment densities and nonnegative lengths required");
  }
  if (!(B->rock_density > 0.0)) return fail(ctx, DP_ERR_ARG, "positive rock density required");
  std::vector<int32_t> valid(nd);
  for (long d = 0; d < nd; ++d) {
    // invalid paths and non-positive cos(zenith) give (NaN, NaN) (src/Tomography.jl:991-993)
    valid[d] = (!B->valid || B->valid[d]) && B->cos_theta[d] > 0.0 ? 1 : 0;
  }
  if (B->energy) {
    for (long i = 0; i < n; ++i)
      if (B->charge[i] != 1.0 && B->charge[i] != -1.0)
        return fail(ctx, DP_ERR_ARG,
                    "MC requires physical charges +-1; CSDA quadrature nodes are not MC samples");
  } else if (!(B->energy_min > 0.0)) {
    return fail(ctx, DP_ERR_ARG, "energy_min must be positive");
  }
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t db = size_t(nd) * 8, sb = size_t(ns) * 8, nb = size_t(n) * 8;
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, 3 * db + 2 * (db + 8) + size_t(nd) * 4 + sb * 2 +
                                               size_t(ns) * 4 + 3 * nb + size_t(nd) * sizeof(dp_los_result) +
                                               16 * 256, 2));
  A.cap = ctx->slot_bytes[2];
  dp_dir_batch D = *B;
  double* ct = A.take<double>(nd);
  double* rr = A.take<double>(nd);
  double* ad = A.take<double>(nd);
  int64_t* sp = A.take<int64_t>(nd + 1);
  int64_t* pp = A.take<int64_t>(nd + 1);
  int32_t* va = A.take<int32_t>(nd);
  int32_t* sm = A.take<int32_t>(ns);
  double* sd = A.take<double>(ns);
  double* sl = A.take<double>(ns);
  double* dE = B->energy ? A.take<double>(n) : nullptr;
  double* dq = B->energy ? A.take<double>(n) : nullptr;
  double* dw = B->energy ? A.take<double>(n) : nullptr;
  dp_los_result* dr = A.take<dp_los_result>(nd);
  if (!dr) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  cudaStream_t s = ctx->stream;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
  };
  cudaError_t e = cudaSuccess;
  for (auto c : {up(ct, B->cos_theta, db), up(rr, B->remaining_rock, db), up(ad, B->air_distance, db),
                 up(sp, B->seg_ptr, db + 8), up(pp, B->sample_ptr, db + 8), up(va, valid.data(), size_t(nd) * 4),
                 up(sm, B->seg_medium, size_t(ns) * 4), up(sd, B->seg_density, sb),
                 up(sl, B->seg_length, sb)})
    if (c != cudaSuccess) e = c;
  if (B->energy)
    for (auto c : {up(dE, B->energy, nb), up(dq, B->charge, nb), up(dw, B->weight, nb)})
      if (c != cudaSuccess) e = c;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpyAsync");
  D.cos_theta = ct;
  D.remaining_rock = rr;
  D.air_distance = ad;
  D.seg_ptr = sp;
  D.sample_ptr = pp;
  D.valid = va;
  D.seg_medium = sm;
  D.seg_density = sd;
  D.seg_length = sl;
  D.energy = dE;
  D.charge = dq;
  D.weight = dw;
  int* bits = nullptr;
  double* dc = nullptr;
  int32_t* dst = nullptr;
  double* dfin = nullptr;
  int rc = dir_run(ctx, ph, M, &D, n, cfg, dr, &bits, &dc, &dst, final_state ? &dfin : nullptr);
  if (rc) return rc;
  if (final_state && n)
    DP_CHECK_CUDA(ctx, cudaMemcpyAsync(final_state, dfin, 2 * nb, cudaMemcpyDeviceToHost, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(out, dr, size_t(nd) * sizeof(dp_los_result), cudaMemcpyDeviceToHost, s));
  if (contrib && n) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(contrib, dc, nb, cudaMemcpyDeviceToHost, s));
  if (status && n) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(status, dst, size_t(n) * 4, cudaMemcpyDeviceToHost, s));
  return status_result(ctx, bits);
}

}  // extern "C"

// mc.cu -- stochastic backward Monte Carlo of libdpgpu: medium preparation on
// the host (mixture properties and the MIXED transport kernel), the
// persistent history kernel in FP64 and mixed precision, the deterministic
// per-line-of-sight tallies and the C ABI.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "mc_host.h"
#include "mc_loop.cuh"

namespace {
// Nuclear RMS radii (fm) by atomic number (src/Straggling.jl:726-729 table).
#include "physics_data.inc"
}  // namespace

using namespace dp;
using namespace dp::mc;

namespace {

std::atomic<uint64_t> g_uid{1};

// interpolate_table_fast (src/Physics.jl:660-687) on the host.
double h_interp(double x, const double* xs, const double* lxs, const double* ys, int n) {
  if (x <= xs[0]) return ys[0];
  if (x >= xs[n - 1]) return ys[n - 1];
  double lx = std::log(x);
  int lo = 0, hi = n - 1;
  while (lo < hi - 1) {
    int mid = (lo + hi) >> 1;
    if (lx < lxs[mid]) hi = mid; else lo = mid;
  }
  double t = (lx - lxs[lo]) / (lxs[lo + 1] - lxs[lo]);
  return ys[lo] + t * (ys[lo + 1] - ys[lo]);
}

const double* hcol(const dp_physics* ph, int mat, int c) {
  return ph->host.data() + (size_t(mat) * DP_NCOL + c) * ph->n;
}

double rms_radius(double Z) {
  long iz = std::lround(Z);
  int i = int(std::min(std::max(iz, 1L), 120L));
  return DPDATA_NUCLEAR_RMS_RADII_FM[i - 1] * 1e-15;
}

int prepare(dp_ctx* ctx, const dp_physics* ph, int nm, const int* mats, const double* fr,
            dp_mixture* m) {
  if (!ph->has_recipes) return fail(ctx, DP_ERR_ARG, "elemental recipes required");
  if (nm < 1 || nm > kMaxMix) return fail(ctx, DP_ERR_ARG, "a mixture holds 1 to 4 materials");
  double tot = 0.0;
  for (int j = 0; j < nm; ++j) {
    if (mats[j] < 0 || mats[j] >= ph->n_mat) return fail(ctx, DP_ERR_ARG, "invalid mixture material");
    if (!(std::isfinite(fr[j]) && fr[j] >= 0.0)) return fail(ctx, DP_ERR_ARG, "invalid mixture fractions");
    tot += fr[j];
  }
  if (!(tot > 0.0)) return fail(ctx, DP_ERR_ARG, "invalid mixture fractions");
  const int n = ph->n;
  const double* E = hcol(ph, mats[0], DP_COL_E);
  const double* lE = hcol(ph, mats[0], DP_COL_LOGE);
  for (int j = 1; j < nm; ++j)
    if (std::memcmp(E, hcol(ph, mats[j], DP_COL_E), sizeof(double) * n) != 0)
      return fail(ctx, DP_ERR_ARG, "mixture materials must share the energy grid");
  m->phys = ph;
  m->uid = g_uid.fetch_add(1);
  m->nm = nm;
  m->mats.assign(mats, mats + nm);
  m->fracs.resize(nm);
  // MaterialMixture normalises its fractions (src/Types.jl:363-368)
  for (int j = 0; j < nm; ++j) m->fracs[j] = fr[j] / tot;
  m->n = n;
  const int ncol = MC_LB1 + 2 * nm;
  m->cols.assign(size_t(ncol) * n, 0.0);
  auto C = [&](int c) { return m->cols.data() + size_t(c) * n; };
  std::copy(E, E + n, C(MC_E));
  std::copy(lE, lE + n, C(MC_LE));
  const int src[7] = {DP_COL_CSDA_S, DP_COL_CSDA_R, DP_COL_MIXED_S, DP_COL_MIXED_R,
                      DP_COL_STRAG, DP_COL_MU0, DP_COL_FSPIN};
  const int dst[7] = {MC_CS, MC_CR, MC_MS, MC_MR, MC_STRAG, MC_MU0, MC_FSPIN};
  if (nm == 1) {
    for (int k = 0; k < 7; ++k) std::copy(hcol(ph, mats[0], src[k]), hcol(ph, mats[0], src[k]) + n, C(dst[k]));
    m->ZoA = ph->recipes[mats[0]].ZoA;
  } else {
    // src/Physics.jl:1152-1323: fraction-weighted node values on the shared
    // grid; ranges integrated from the mixture stopping power
    // (_build_mixture_table, src/Physics.jl:1058-1105)
    for (int k = 0; k < 7; ++k) {
      if (dst[k] == MC_CR || dst[k] == MC_MR) continue;
      double* o = C(dst[k]);
      for (int j = 0; j < nm; ++j) {
        const double* y = hcol(ph, mats[j], src[k]);
        for (int i = 0; i < n; ++i) o[i] += m->fracs[j] * y[i];
      }
    }
    const double* gE = hcol(ph, 0, DP_COL_E);
    auto stop = [&](bool mixed, double K) {
      double v = 0.0;
      for (int j = 0; j < nm; ++j)
        v += m->fracs[j] * h_interp(K, hcol(ph, mats[j], DP_COL_E), hcol(ph, mats[j], DP_COL_LOGE),
                                    hcol(ph, mats[j], mixed ? DP_COL_MIXED_S : DP_COL_CSDA_S), n);
      return v;
    };
    double* cR = C(MC_CR);
    double* mR = C(MC_MR);
    double cp = stop(false, gE[0]), mp = stop(true, gE[0]);
    cR[0] = gE[0] / cp;
    mR[0] = gE[0] / mp;
    for (int i = 1; i < n; ++i) {
      double K = gE[i], Kp = gE[i - 1], dK = K - Kp;
      double c = stop(false, K), mm = stop(true, K);
      cR[i] = cR[i - 1] + dK / ((c + cp) / 2);
      mR[i] = mR[i - 1] + dK / ((mm + mp) / 2);
      cp = c;
      mp = mm;
    }
    m->ZoA = 0.0;
    for (int j = 0; j < nm; ++j) m->ZoA += m->fracs[j] * ph->recipes[mats[j]].ZoA;
  }
  for (int j = 0; j < nm; ++j) {
    std::copy(hcol(ph, mats[j], DP_COL_LB1), hcol(ph, mats[j], DP_COL_LB1) + n, C(MC_LB1 + j));
    std::copy(hcol(ph, mats[j], DP_COL_LBE), hcol(ph, mats[j], DP_COL_LBE) + n, C(MC_LB1 + nm + j));
  }

  // prepare_mixed_kernel (src/MixedTransport.jl:57-97)
  const dp_settings& st = ph->settings;
  double lo = -1e300, hi = 1e300;
  for (int j = 0; j < nm; ++j) {
    lo = std::max(lo, hcol(ph, mats[j], DP_COL_E)[0]);
    hi = std::min(hi, hcol(ph, mats[j], DP_COL_E)[n - 1]);
  }
  std::vector<double> grid;
  for (int j = 0; j < nm; ++j)
    for (int i = 0; i < n; ++i) {
      double e = hcol(ph, mats[j], DP_COL_E)[i];
      if (lo <= e && e <= hi) grid.push_back(e);
    }
  std::sort(grid.begin(), grid.end());
  grid.erase(std::unique(grid.begin(), grid.end()), grid.end());
  const int refinement = 8;
  std::vector<double> kE;
  for (size_t j = 0; j + 1 < grid.size(); ++j) {
    double a = std::log(grid[j]), b = std::log(grid[j + 1]);
    for (int k = 0; k < refinement; ++k)
      kE.push_back(std::exp(a + double(k) * (b - a) / double(refinement)));
  }
  kE.push_back(hi);
  kE[0] = lo;
  const int nk = int(kE.size());
  auto prop = [&](int col, double k) {
    double v = 0.0;
    for (int j = 0; j < nm; ++j)
      v += m->fracs[j] * h_interp(k, hcol(ph, mats[j], DP_COL_E), hcol(ph, mats[j], DP_COL_LOGE),
                                  hcol(ph, mats[j], col), n);
    return v;
  };
  m->nk = nk;
  m->kcols.assign(size_t(K_NCOL) * nk, 0.0);
  double* K0 = m->kcols.data();
  double *kS = K0 + size_t(K_S) * nk, *kSig = K0 + size_t(K_SIG) * nk,
         *kR = K0 + size_t(K_R) * nk, *kH = K0 + size_t(K_H) * nk, *kT = K0 + size_t(K_T) * nk;
  std::copy(kE.begin(), kE.end(), K0);
  for (int i = 0; i < nk; ++i) {
    kS[i] = prop(DP_COL_MIXED_S, kE[i]);
    kSig[i] = prop(DP_COL_XS, kE[i]);
  }
  m->onset = std::numeric_limits<double>::infinity();
  for (double g : grid) {
    double r = prop(DP_COL_XS, g);
    if (r > 0) {
      m->onset = g;
      for (int i = 0; i < nk; ++i)
        if (kE[i] < g) kSig[i] = r;
      break;
    }
  }
  for (int j = 1; j < nk; ++j) {
    double a = kE[j - 1], b = kE[j], d = b - a;
    kR[j] = kR[j - 1] + d / 2 * (1 / kS[j - 1] + 1 / kS[j]);
    kH[j] = kH[j - 1] + d / 2 * (kSig[j - 1] / kS[j - 1] + kSig[j] / kS[j]);
    kT[j] = kT[j - 1] + d / 2 * st.mass *
                            (1 / (std::sqrt(a * (a + 2 * st.mass)) * kS[j - 1]) +
                             1 / (std::sqrt(b * (b + 2 * st.mass)) * kS[j]));
  }
  m->el.clear();
  for (int j = 0; j < nm; ++j)
    for (const HostElement& e : ph->recipes[mats[j]].elements) {
      const double v[kElStride] = {e.Z, e.A, e.I, m->fracs[j] * e.fraction, rms_radius(e.Z)};
      m->el.insert(m->el.end(), v, v + kElStride);
    }
  m->nel = int(m->el.size() / kElStride);
  if (m->nel > kMaxEl) return fail(ctx, DP_ERR_ARG, "a medium holds at most 32 elements");
  return DP_OK;
}

int pad_elems(int n, size_t esize) {
  int per = int(16 / esize);
  return (n + per - 1) / per * per;
}

}  // namespace

namespace dp {
namespace mc {

Layout make_layout(const dp_mixture* const* media, int n_media, size_t esize) {
  const dp_mixture* a = media[0];
  Layout L{};
  L.n = a->n;
  L.nk = a->nk;
  L.slots = 1;
  bool same_nk = true;
  for (int k = 0; k < n_media; ++k) {
    L.slots = std::max(L.slots, media[k]->nm);
    same_nk = same_nk && media[k]->nk == a->nk;
  }
  L.ld = pad_elems(L.n, esize);
  L.ldk = pad_elems(L.nk, esize);
  // elements, then the index-table origins and widths (2 doubles per column)
  L.o_phys = uint32_t((kMaxEl * kElStride + 2 * I_NCOL) * sizeof(double));
  L.o_ker = L.o_phys + uint32_t(size_t(MC_LB1 + 2 * L.slots) * L.ld * esize);
  L.o_idx = L.o_ker + uint32_t(size_t(K_NCOL) * L.ldk * esize);
  L.nbp = kIdxBinsPhys;
  L.nbk = kIdxBinsKer;
  uint32_t idx_bytes = uint32_t((2 * kIdxBinsPhys + 2 * kIdxBinsKer) * sizeof(int16_t));
  L.o_elf = L.o_idx + (idx_bytes + 15) / 16 * 16;
  L.med_bytes = L.o_elf + uint32_t(kMaxEl * kElfStride * sizeof(float));
  const dp_physics* ph = a->phys;
  L.uniform = ph->view.uniform;
  L.lE0 = ph->view.lE0;
  L.inv_dlE = ph->view.inv_dlE;
  // kernel energies: 8 log-uniform nodes per interval of a uniform grid
  L.kuniform = L.uniform && a->nk == 8 * (a->n - 1) + 1 && same_nk ? 1 : 0;
  L.kinv_dlE = 8.0 * ph->view.inv_dlE;
  return L;
}

template <class R>
static void pack(const dp_mixture* m, const Layout& L, unsigned char* out) {
  std::memset(out, 0, L.med_bytes);
  std::memcpy(out, m->el.data(), m->el.size() * sizeof(double));
  R* P = reinterpret_cast<R*>(out + L.o_phys);
  auto put = [&](R* dst, const double* src, int n) {
    for (int i = 0; i < n; ++i) dst[i] = R(src[i]);
  };
  for (int c = 0; c < MC_LB1; ++c) put(P + size_t(c) * L.ld, m->cols.data() + size_t(c) * m->n, m->n);
  for (int j = 0; j < m->nm; ++j) {
    put(P + size_t(MC_LB1 + j) * L.ld, m->cols.data() + size_t(MC_LB1 + j) * m->n, m->n);
    put(P + size_t(MC_LB1 + L.slots + j) * L.ld, m->cols.data() + size_t(MC_LB1 + m->nm + j) * m->n,
        m->n);
  }
  R* K = reinterpret_cast<R*>(out + L.o_ker);
  for (int c = 0; c < K_NCOL; ++c) put(K + size_t(c) * L.ldk, m->kcols.data() + size_t(c) * m->nk, m->nk);
  // FP32 element table of the cooperative DCS sums
  float* elf = reinterpret_cast<float*>(out + L.o_elf);
  for (int e = 0; e < m->nel; ++e) {
    const double* x = m->el.data() + kElStride * e;
    float* f = elf + kElfStride * e;
    f[0] = float(x[0]);
    f[1] = float(x[1]);
    f[2] = float(x[2]);
    f[3] = float(x[3]);
    f[4] = float(kAvogadro / (x[1] * 0.001));
    f[5] = float(x[4]);  // nuclear RMS radius (DEL polar angles)
  }
  // index tables of the inverse lookups (origins and widths in R)
  R* prm = reinterpret_cast<R*>(reinterpret_cast<double*>(out) + kMaxEl * kElStride);
  int16_t* idx = reinterpret_cast<int16_t*>(out + L.o_idx);
  const double* cols[I_NCOL] = {m->cols.data() + size_t(MC_CR) * m->n,
                                m->cols.data() + size_t(MC_MR) * m->n,
                                m->kcols.data() + size_t(K_R) * m->nk,
                                m->kcols.data() + size_t(K_H) * m->nk};
  for (int c = 0; c < I_NCOL; ++c) {
    const int n = c < I_KR ? m->n : m->nk, nb = c < I_KR ? kIdxBinsPhys : kIdxBinsKer;
    int16_t* out_idx = idx + (c < I_KR ? c * kIdxBinsPhys : 2 * kIdxBinsPhys + (c - I_KR) * kIdxBinsKer);
    const double* y = cols[c];
    int j0 = 0;
    while (j0 < n - 1 && !(y[j0] > 0.0)) ++j0;
    double lo = y[j0] > 0.0 ? std::log(y[j0]) : 0.0;
    double hi = y[n - 1] > 0.0 ? std::log(y[n - 1]) : lo;
    double inv = hi > lo ? nb / (hi - lo) : 0.0;
    prm[2 * c] = R(lo);
    prm[2 * c + 1] = R(inv);
    int j = 0;
    for (int b = 0; b < nb; ++b) {
      double edge = inv > 0.0 ? std::exp(lo + b / inv) : 0.0;
      while (j < n - 2 && y[j + 1] <= edge) ++j;
      out_idx[b] = int16_t(j);
    }
  }
}

void pack_medium(const dp_mixture* m, const Layout& L, size_t esize, unsigned char* out) {
  if (esize == sizeof(float)) pack<float>(m, L, out);
  else pack<double>(m, L, out);
}

MedInfo make_info(const dp_mixture* m) {
  MedInfo I{};
  I.nm = m->nm;
  I.nel = m->nel;
  for (int j = 0; j < kMaxMix; ++j) I.frac[j] = j < m->nm ? m->fracs[j] : 0.0;
  I.ZoA = m->ZoA;
  I.onset = m->onset;
  return I;
}

}  // namespace mc
}  // namespace dp

namespace {

// Device blob of the (rock, air[, porous]) media in one precision, built
// once per combination.
int get_blob(dp_ctx* ctx, dp_mixture* rock, const dp_mixture* air, int precision,
             const unsigned char** dev, Layout* lay, const dp_mixture* porous = nullptr) {
  const uint64_t puid = porous ? porous->uid : 0;
  for (auto& b : rock->blobs)
    if (b.partner == air->uid && b.partner2 == puid && b.precision == precision) {
      *dev = b.dev;
      *lay = b.lay;
      return DP_OK;
    }
  if (rock->n != air->n || rock->nk != air->nk || rock->phys != air->phys ||
      (porous && (porous->n != rock->n || porous->nk != rock->nk || porous->phys != rock->phys)))
    return fail(ctx, DP_ERR_ARG, "rock, air and porous media must come from one physics");
  size_t es = precision == DP_PREC_MIXED ? sizeof(float) : sizeof(double);
  const dp_mixture* media[3] = {rock, air, porous};
  const int nm = porous ? 3 : 2;
  Layout L = make_layout(media, nm, es);
  std::vector<unsigned char> h(size_t(nm) * L.med_bytes);
  for (int k = 0; k < nm; ++k) pack_medium(media[k], L, es, h.data() + size_t(k) * L.med_bytes);
  unsigned char* d = nullptr;
  DP_CHECK_CUDA(ctx, cudaMalloc(&d, h.size()));
  DP_CHECK_CUDA(ctx, cudaMemcpy(d, h.data(), h.size(), cudaMemcpyHostToDevice));
  rock->blobs.push_back({air->uid, puid, precision, d, L});
  *dev = d;
  *lay = L;
  return DP_OK;
}

}  // namespace

// ------------------------------------------------------------------ kernel
namespace dp {
namespace mc {

struct McParams {
  const unsigned char* blob;  // rock medium, air medium, then the porous medium if any
  Layout lay;
  MedInfo info[3];
  int porous;                 // the columns have a porous top layer (porous_rec)
  Consts C;
  uint64_t seed;
  int staged;
  int source;  // 0 explicit histories, 1 lines of sight
  long n;
  uint64_t id0;
  const double *E, *q, *w, *thick, *dens, *elev, *H;
  int geo_stride;
  const dp_los* los;
  const int64_t* los_off;  // n_los + 1 running sample offsets
  long n_los;
  double* contrib;
  int32_t* status;
  int32_t* steps;
  double* efinal;
  unsigned long long* counter;  // [0] phase-0 histories taken, [1] phase-1, [2] queued
  int* err_flag;
  int coop_nel, coop_stride, coop_kmax;  // batched DCS buffers: elements, floats per warp, events
  int coop_kc;  // events per chunk of the CTA buffer (lockstep phases)
  int sync;     // bit k: phase k runs its steps in CTA lockstep
  void* queue;                // Handoff<R> x n: histories crossing the mode switch
  void* start;                // StartRec<R> x n
  void* end;                  // EndRec<R> x n
  void* porous_rec;           // PorousRec<R> x n when porous
  // longest-first schedule (null: counter order): per history the cost
  // buckets of its phase-0 and phase-1 work, the hand-out orders (history
  // indices, queue slots) and 2 x kSchedBuckets words of counting-sort scratch
  uint16_t *key0, *key1;
  uint32_t *order0, *order1, *sched;
};

// Cost buckets of a history for the longest-first schedule.  Phase 0 (below
// the mode switch): its step count follows log(1 + G / X0), G the rock
// grammage along the direction and X0 the CSDA range at the start energy
// (the step limits are a fixed fraction of the range), 64 buckets per unit.
// Phase 1 (mixed steps from hard event to hard event): it follows the rock
// grammage left above the switch, log(1 + G1 / 1e4 kg/m^2), 128 buckets per
// unit.  A history above the switch at the start costs phase 0 nothing.
template <class R>
__device__ __forceinline__ void cost_buckets(const Med<R>& rock, const Consts& C, double E0,
                                             double thick, double rho, double uz, uint16_t* k0,
                                             uint16_t* k1) {
  const double G = thick * rho / fmax(fabs(uz), 0.05);
  const double X0 = double(at(rock, locate(rock, R(E0)), MC_CR));
  const double Xs = double(at(rock, locate(rock, R(C.thr_low)), MC_CR));
  const double G1 = fmax(G - fmax(Xs - X0, 0.0), 0.0);
  const double c0 = E0 < C.thr_low ? log1p(G / fmax(X0, 1e-3)) * 64.0 : 0.0;
  const double c1 = log1p(G1 * 1e-4) * 128.0;
  *k0 = uint16_t(fmin(c0, double(kSchedBuckets - 1)));
  *k1 = uint16_t(fmin(c1, double(kSchedBuckets - 1)));
}
struct KeyOf {
  const uint16_t* key;
  __device__ int operator()(long s) const { return key[s]; }
};
template <class Q>
struct QueueKeyOf {
  const Q* queue;
  const uint16_t* key;
  __device__ int operator()(long s) const { return key[queue[s].index]; }
};

// Start record of history i: energy, charge and weight drawn as
// run_backward_mc draws them (src/Geometry.jl:863-875) or given; geometry
// given, taken from its line of sight or drawn (Philox blocks 1-2).
template <class R>
__global__ void __launch_bounds__(256) mc_init_kernel(const __grid_constant__ McParams P) {
  StartRec<R>* out = static_cast<StartRec<R>*>(P.start);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < P.n;
       i += long(gridDim.x) * blockDim.x) {
    double E0, q, ws, thick, rho, elev, H, p_thick = 0.0, p_rho = 0.0;
    if (P.source == 0) {
      E0 = P.E[i];
      q = P.q[i];
      ws = P.w[i];
      long gi = P.geo_stride ? i : 0;
      thick = P.thick[gi];
      rho = P.dens[gi];
      elev = P.elev[gi];
      H = P.H[gi];
    } else {
      long lo = 0, hi = P.n_los;  // los_off[lo] <= i < los_off[lo + 1]
      while (hi - lo > 1) {
        long mid = (lo + hi) >> 1;
        if (P.los_off[mid] <= i) lo = mid; else hi = mid;
      }
      const dp_los& L = P.los[lo];
      const uint64_t id = uint64_t(i);
      double emax = L.energy_max > L.energy_min ? L.energy_max : L.energy_min;
      mc_sample(P.seed, id, L.energy_min, emax, &E0, &q, &ws);
      U4 b1 = philox(U4{uint32_t(id), uint32_t(id >> 32), 1u, 0u}, uint32_t(P.seed),
                     uint32_t(P.seed >> 32));
      U4 b2 = philox(U4{uint32_t(id), uint32_t(id >> 32), 2u, 0u}, uint32_t(P.seed),
                     uint32_t(P.seed >> 32));
      thick = L.thickness_max > L.thickness
                  ? L.thickness + (L.thickness_max - L.thickness) * u01(b1.x, b1.y)
                  : L.thickness;
      rho = L.density_max > L.density ? L.density + (L.density_max - L.density) * u01(b1.z, b1.w)
                                      : L.density;
      elev = L.elevation_max > L.elevation
                 ? L.elevation + (L.elevation_max - L.elevation) * u01(b2.x, b2.y)
                 : L.elevation;
      H = L.air_height > 0.0 ? thick + L.air_height
                             : (L.primary_altitude > 0.0 ? L.primary_altitude : 3e4);
      p_thick = L.porous_thickness;
      p_rho = L.porous_density;
    }
    if (P.porous) {
      // porous_z = rock_thickness - porous_thickness when the layer is
      // present (src/Geometry.jl:617-618), else the rock top
      PorousRec<R> pr;
      pr.pz = alt_make<R>(p_thick > 0.0 ? thick - p_thick : thick);
      pr.prho = R(p_rho);
      static_cast<PorousRec<R>*>(P.porous_rec)[i] = pr;
    }
    double theta = (90.0 - elev) * kPi / 180.0;
    if (P.key0) {
      const Med<R> rock = make_med<R>(P.blob, P.lay, P.info[0]);
      cost_buckets<R>(rock, P.C, E0, thick, rho, cos(theta), P.key0 + i, P.key1 + i);
    }
    StartRec<R> r;
    r.thick = alt_make<R>(thick);
    r.H = alt_make<R>(H);
    r.q = q;
    r.ws = ws;
    r.E = R(E0);
    r.rho = R(rho);
    r.ux = R(-sin(theta));
    r.uz = R(-cos(theta));
    out[i] = r;
  }
}

template <class R>
__device__ __forceinline__ void start_history(const McParams& P, long i, Hist<R>& h, Stream& g) {
  const StartRec<R> r = static_cast<const StartRec<R>*>(P.start)[i];
  h.s.z = alt_make<R>(0.0);
  h.s.ux = r.ux;
  h.s.uy = R(0);
  h.s.uz = r.uz;
  h.s.E = r.E;
  h.s.w = R(1);
  h.s.status = 0;
  h.limit = R(0);
  h.thick = r.thick;
  h.rho = r.rho;
  h.H = r.H;
  h.steps = h.inner = h.outer = 0;
  h.need_mode = true;
  h.strag = h.mixed = h.scat = false;
  h.x.kind = CONT_NONE;
  g.init(P.seed, P.source == 0 ? P.id0 + uint64_t(i) : uint64_t(i));
}

template <class R>
__device__ __forceinline__ void end_history(const McParams& P, long i, const Hist<R>& h) {
  EndRec<R> e;
  e.z = h.s.z;
  e.E = h.s.E;
  e.w = h.s.w;
  e.uz = h.s.uz;
  e.status = h.s.status;
  e.steps = h.steps;
  static_cast<EndRec<R>*>(P.end)[i] = e;
}

// Flux contribution w_i * flux_i of every ended history, FP64, one thread per
// history (src/Geometry.jl:729-757).
template <class R>
__global__ void __launch_bounds__(256) mc_finish_kernel(const __grid_constant__ McParams P) {
  const StartRec<R>* st = static_cast<const StartRec<R>*>(P.start);
  const EndRec<R>* en = static_cast<const EndRec<R>*>(P.end);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < P.n;
       i += long(gridDim.x) * blockDim.x) {
    const EndRec<R> e = en[i];
    const StartRec<R> r = st[i];
    P.contrib[i] = r.ws * history_flux(P.C, e, alt_value(r.H), r.q);
    if (P.status) P.status[i] = e.status;
    if (P.steps) P.steps[i] = e.steps;
    if (P.efinal) {
      double* f = P.efinal + 4 * i;
      f[0] = double(e.E);
      f[1] = alt_value(e.z);
      f[2] = double(e.uz);
      f[3] = double(e.w);
    }
  }
}

// Two-layer geometry of run_backward_mc (rock column under air) for the
// shared history loop.
template <class R>
struct SlabGeo {
  using Hist = mc::Hist<R>;
  using Queue = Handoff<R>;
  const McParams& P;
  const Med<R>& rock;
  const Med<R>& air;
  __device__ long n0() const { return P.n; }
  __device__ void start(long i, Hist& h, Stream& g) const { start_history(P, i, h, g); }
  __device__ long load(const Queue& q, Hist& h, Stream& g) const {
    return load_handoff(q, P.seed, h, g);
  }
  __device__ void save(const Hist& h, const Stream& g, long i, Queue* q) const {
    save_handoff(h, g, i, q);
  }
  __device__ void end(long i, const Hist& h) const { end_history(P, i, h); }
  __device__ const Med<R>& medium(int k) const { return k ? air : rock; }
  // the descriptors by medium index: rock and air are consecutive entries of
  // the CTA's descriptor array in shared memory
  __device__ const Med<R>* media() const { return &rock; }
  template <bool COOP, int PHASE>
  __device__ int advance(Hist& h, Stream& g) const {
    return mc::advance<R, COOP, PHASE>(rock, air, nullptr, P.C, h, g);
  }
  template <int PHASE>
  __device__ int resume(Hist& h, Stream& g) const {
    return mc::resume<R, PHASE>(rock, air, nullptr, P.C, h, g);
  }
};

// The same column with the shallow porous top layer (medium 2).
template <class R>
struct SlabGeoP {
  using Hist = mc::HistP<R>;
  using Queue = HandoffP<R>;
  const McParams& P;
  const Med<R>& rock;
  const Med<R>& air;
  const Med<R>& porous;
  __device__ long n0() const { return P.n; }
  __device__ void start(long i, Hist& h, Stream& g) const {
    start_history(P, i, h, g);
    const PorousRec<R> pr = static_cast<const PorousRec<R>*>(P.porous_rec)[i];
    h.pz = pr.pz;
    h.prho = pr.prho;
  }
  __device__ long load(const Queue& q, Hist& h, Stream& g) const {
    const long i = load_handoff(q, P.seed, h, g);
    h.pz = q.pz;
    h.prho = q.prho;
    return i;
  }
  __device__ void save(const Hist& h, const Stream& g, long i, Queue* q) const {
    save_handoff(h, g, i, q);
    q->pz = h.pz;
    q->prho = h.prho;
  }
  __device__ void end(long i, const Hist& h) const { end_history(P, i, h); }
  __device__ const Med<R>& medium(int k) const { return k == 1 ? air : (k == 2 ? porous : rock); }
  // rock, air and porous are consecutive entries of the CTA's descriptor array
  __device__ const Med<R>* media() const { return &rock; }
  template <bool COOP, int PHASE>
  __device__ int advance(Hist& h, Stream& g) const {
    return mc::advance<R, COOP, PHASE>(rock, air, &porous, P.C, h, g);
  }
  template <int PHASE>
  __device__ int resume(Hist& h, Stream& g) const {
    return mc::resume<R, PHASE>(rock, air, &porous, P.C, h, g);
  }
};

// Shared-memory header of the transport kernels: the staging mbarrier, then
// the medium descriptors (rock, air, porous), one copy per CTA: the helpers
// that take a medium by reference then read it there instead of from a copy
// in every thread's stack.
template <class R>
constexpr size_t mc_smem_head() {
  return (16 + 3 * sizeof(Med<R>) + 15) / 16 * 16;
}

template <class R, int PHASE, int T, bool POR = false>
__global__ void __launch_bounds__(T, 1) mc_kernel(const __grid_constant__ McParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr size_t head = mc_smem_head<R>();
  const unsigned char* base = P.blob;
  const uint32_t tables = P.staged ? (POR ? 3 : 2) * P.lay.med_bytes : 0;
  if (P.staged) {
    if (!stage_blob(smem + head, P.blob, tables, reinterpret_cast<uint64_t*>(smem), P.C.wait_iters)) {
      if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
      const Med<R> none{};
      if constexpr (POR) {
        SlabGeoP<R> geo{P, none, none, none};
        drain_histories<R, PHASE>(geo, P.counter, static_cast<HandoffP<R>*>(P.queue),
                                  PHASE == 0 ? P.order0 : P.order1);
      } else {
        SlabGeo<R> geo{P, none, none};
        drain_histories<R, PHASE>(geo, P.counter, static_cast<Handoff<R>*>(P.queue),
                                  PHASE == 0 ? P.order0 : P.order1);
      }
      return;
    }
    base = smem + head;
  }
  Med<R>* meds = reinterpret_cast<Med<R>*>(smem + 16);
  if (threadIdx.x < (POR ? 3 : 2))
    meds[threadIdx.x] = make_med<R>(base + threadIdx.x * P.lay.med_bytes, P.lay, P.info[threadIdx.x]);
  __syncthreads();
  const Med<R>& rock = meds[0];
  const Med<R>& air = meds[1];
  float* coop = reinterpret_cast<float*>(smem + head + tables);
  if constexpr (POR) {
    const Med<R>& porous = meds[2];
    SlabGeoP<R> geo{P, rock, air, porous};
    transport_histories<R, PHASE, KCfg<R>::coop>(geo, P.C, P.counter,
                                                 static_cast<HandoffP<R>*>(P.queue), coop,
                                                 P.coop_stride, P.coop_kmax, P.coop_kc, P.coop_nel,
                                                 PHASE == 0 ? P.order0 : P.order1,
                                                 ((P.sync >> PHASE) & 1) != 0);
  } else {
    SlabGeo<R> geo{P, rock, air};
    transport_histories<R, PHASE, KCfg<R>::coop>(geo, P.C, P.counter,
                                                 static_cast<Handoff<R>*>(P.queue), coop,
                                                 P.coop_stride, P.coop_kmax, P.coop_kc, P.coop_nel,
                                                 PHASE == 0 ? P.order0 : P.order1,
                                                 ((P.sync >> PHASE) & 1) != 0);
  }
}

// Per line of sight: compensated sums of the contributions and of their
// squares in a fixed order, then flux, sigma (src/Geometry.jl:883-893) and
// the count of flagged histories.  Two levels so that one long line of sight
// does not serialise on one warp: fixed chunks of kTallyChunk histories of a
// line (one warp each), then one warp per line combines its chunks in order.
constexpr long kTallyChunk = 4096;
struct TallyPart {
  KSum s, s2, gf, g;
  long bad;
  int bits;
};
__device__ __forceinline__ void warp_down(KSum& v, int d) {
  KSum o{__shfl_down_sync(0xffffffffu, v.s, d), __shfl_down_sync(0xffffffffu, v.c, d)};
  kmerge(v, o);
}
__global__ void __launch_bounds__(256) los_chunk_kernel(const double* contrib, const int32_t* status,
                                                        const int64_t* off, const int64_t* coff,
                                                        long n_los, long max_jobs,
                                                        const double* csda, const double* dcsda,
                                                        TallyPart* part) {
  long j = (long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (j >= max_jobs || j >= coff[n_los]) return;
  long lo = 0, hi = n_los;  // coff[lo] <= j < coff[lo + 1]
  while (hi - lo > 1) {
    long mid = (lo + hi) >> 1;
    if (coff[mid] <= j) lo = mid; else hi = mid;
  }
  const long a = off[lo] + (j - coff[lo]) * kTallyChunk;
  const long b = a + kTallyChunk < off[lo + 1] ? a + kTallyChunk : off[lo + 1];
  TallyPart t{{0, 0}, {0, 0}, {0, 0}, {0, 0}, 0, 0};
  for (long i = a + lane; i < b; i += 32) {
    double x = contrib[i];
    kadd(t.s, x);
    kadd(t.s2, x * x);
    int st = status[i];
    t.bad += st != 0;
    t.bits |= st;
    if (csda) {
      kadd(t.gf, csda[i]);
      kadd(t.g, dcsda[i]);
    }
  }
  t.bits = __reduce_or_sync(0xffffffffu, unsigned(t.bits));
  for (int d = 16; d > 0; d >>= 1) {
    warp_down(t.s, d);
    warp_down(t.s2, d);
    warp_down(t.gf, d);
    warp_down(t.g, d);
    t.bad += __shfl_down_sync(0xffffffffu, t.bad, d);
  }
  if (lane == 0) part[j] = t;
}
// sigma_n1 = 0: run_backward_mc's sigma (src/Geometry.jl:883-893); 1: the
// directional MC's, with n - 1 (src/Tomography.jl:1036-1039), NaN results
// for directions with valid[l] == 0 (src/Tomography.jl:991-993).
__global__ void __launch_bounds__(256) los_tally_kernel(const TallyPart* part, const int64_t* off,
                                                        const int64_t* coff, const dp_los* los,
                                                        const int32_t* valid, long n_los,
                                                        int has_csda, int sigma_n1,
                                                        dp_los_result* out, int* status_or) {
  long l = (long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (l >= n_los) return;
  TallyPart t{{0, 0}, {0, 0}, {0, 0}, {0, 0}, 0, 0};
  for (int64_t j = coff[l] + lane; j < coff[l + 1]; j += 32) {
    const TallyPart& q = part[j];
    kmerge(t.s, q.s);
    kmerge(t.s2, q.s2);
    kmerge(t.gf, q.gf);
    kmerge(t.g, q.g);
    t.bad += q.bad;
    t.bits |= q.bits;
  }
  t.bits = __reduce_or_sync(0xffffffffu, unsigned(t.bits));
  for (int d = 16; d > 0; d >>= 1) {
    warp_down(t.s, d);
    warp_down(t.s2, d);
    warp_down(t.gf, d);
    warp_down(t.g, d);
    t.bad += __shfl_down_sync(0xffffffffu, t.bad, d);
  }
  if (lane == 0) {
    long n = off[l + 1] - off[l];
    double sum = t.s.s + t.s.c, sum2 = t.s2.s + t.s2.c;
    dp_los_result r{};
    r.n_samples = n;
    r.n_status_nonzero = t.bad;
    if (n > 0) {
      double f = sum / double(n), var = sum2 / double(n) - f * f;
      r.flux = f;
      if (sigma_n1) r.sigma = sqrt(fmax(0.0, var / double(n > 1 ? n - 1 : 1)));
      else r.sigma = los[l].thickness > 0.0 ? sqrt(fmax(var, 0.0) / double(n)) : 0.0;
      if (has_csda) {
        r.gradient_flux = (t.gf.s + t.gf.c) / double(n);
        r.gradient = (t.g.s + t.g.c) / double(n);
      }
    }
    if (valid && !valid[l]) r.flux = r.sigma = CUDART_NAN;
    out[l] = r;
    if (t.bits) atomicOr(status_or, t.bits);
  }
}

// Running sample offsets of the lines of sight (single block, sequential
// chunks; n_los is at most a few 10^5), or a copy of given offsets, and the
// running chunk offsets of the tally (coff).
__global__ void __launch_bounds__(1024) los_offsets_kernel(const dp_los* los, const int64_t* given,
                                                           long n_los, int64_t* off, int64_t* coff,
                                                           long expect, int* err) {
  __shared__ int64_t part[1024], cpart[1024];
  long per = (n_los + 1023) / 1024;
  long a = threadIdx.x * per, b = a + per < n_los ? a + per : n_los;
  auto count = [&](long l) {
    if (given) return given[l + 1] - given[l] > 0 ? given[l + 1] - given[l] : int64_t(0);
    return los[l].n_samples > 0 ? int64_t(los[l].n_samples) : int64_t(0);
  };
  int64_t s = 0, cs = 0;
  for (long l = a; l < b; ++l) {
    s += count(l);
    cs += (count(l) + kTallyChunk - 1) / kTallyChunk;
  }
  part[threadIdx.x] = s;
  cpart[threadIdx.x] = cs;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0, crun = 0;
    for (int t = 0; t < 1024; ++t) {
      int64_t v = part[t], cv = cpart[t];
      part[t] = run;
      cpart[t] = crun;
      run += v;
      crun += cv;
    }
    off[n_los] = run;
    coff[n_los] = crun;
    if (run != expect) atomicExch(err, 2);
  }
  __syncthreads();
  int64_t run = part[threadIdx.x], crun = cpart[threadIdx.x];
  for (long l = a; l < b; ++l) {
    off[l] = run;
    coff[l] = crun;
    run += count(l);
    crun += (count(l) + kTallyChunk - 1) / kTallyChunk;
  }
}

}  // namespace mc
}  // namespace dp

namespace {

// Per-history device records of a run (hand-off, start, end), sized for FP64.
constexpr size_t kRecBytes = sizeof(HandoffP<double>) + sizeof(StartRec<double>) +
                             sizeof(EndRec<double>) + sizeof(PorousRec<double>) + 64;
// The longest-first schedule: two cost buckets and two order entries per
// history, and the counting-sort words (kSchedExtra covers those and the
// arena's alignment of the five arrays).
constexpr size_t kSchedBytes = 2 * sizeof(uint16_t) + 2 * sizeof(uint32_t);
constexpr size_t kSchedExtra = 2 * kSchedBuckets * sizeof(uint32_t) + 5 * 256;

// Takes the schedule's arrays from the arena when the context hands
// histories out longest first (and the indices fit 32 bits).
void take_sched(dp_ctx* ctx, int precision, long n, Arena& A, McParams& P) {
  if (ctx->mc_order[DP_KERNEL_MC][precision] != 0 || n >= (1L << 32)) return;
  P.key0 = A.take<uint16_t>(n);
  P.key1 = A.take<uint16_t>(n);
  P.order0 = A.take<uint32_t>(n);
  P.order1 = A.take<uint32_t>(n);
  P.sched = A.take<uint32_t>(2 * kSchedBuckets);
  if (!P.sched) P.key0 = P.key1 = nullptr, P.order0 = P.order1 = P.sched = nullptr;
}

}  // namespace

namespace dp {
namespace mc {

int check_cfg(dp_ctx* ctx, const dp_physics* ph, const dp_mc_config* cfg, Consts* C,
              double* thr_fp64) {
  if (!cfg) return fail(ctx, DP_ERR_ARG, "null config");
  if (cfg->precision != DP_PREC_FP64 && cfg->precision != DP_PREC_MIXED)
    return fail(ctx, DP_ERR_ARG, "precision must be DP_PREC_FP64 or DP_PREC_MIXED");
  double tmax = ph->host[(size_t(0) * DP_NCOL + DP_COL_E) * ph->n + ph->n - 1];
  double thr = cfg->source_energy_max > 0.0 ? cfg->source_energy_max : std::fmin(1e9, tmax);
  if (!(thr > 0.0 && thr <= tmax))
    return fail(ctx, DP_ERR_ARG, "source_energy_max must be positive and within the physics energy grid");
  double low = cfg->energy_threshold_low > 0.0 ? cfg->energy_threshold_low : 100.0;
  if (thr_fp64) *thr_fp64 = thr;
  if (cfg->precision == DP_PREC_MIXED) {
    // thresholds exactly representable in the FP32 transport
    thr = double(float(thr));
    if (thr > tmax) thr = double(std::nextafter(float(tmax), 0.0f));
    low = double(float(low));
  }
  C->mass = ph->settings.mass;
  C->ctau = ph->settings.ctau;
  C->cutoff = ph->settings.cutoff;
  C->elastic_ratio = ph->settings.elastic_ratio;
  C->thr = thr;
  C->thr_low = low;
  C->thr_f = float(thr);
  C->thr_low_f = float(low);
  C->mass_f = float(C->mass);
  C->ctau_f = float(C->ctau);
  C->elastic_ratio_f = float(C->elastic_ratio);
  C->cutoff_f = float(C->cutoff);
  C->lcut_f = float(-std::log(C->cutoff));
  C->step_cap = step_cap(ctx);
  C->event_cap = event_cap(ctx);
  C->wait_iters = stage_wait(ctx);
  C->straggling = cfg->straggling != 0;
  C->scattering = cfg->scattering != 0;
  return DP_OK;
}

int read_flag(dp_ctx* ctx) {
  int flag = 0;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
    return fail(ctx, DP_ERR_STATE,
                flag == 2   ? "total_samples differs from the sum of n_samples"
                : flag == 4 ? "a CSDA history reached the transport step cap"
                            : "a table-staging wait exceeded its limit");
  }
  return DP_OK;
}

// The reference's message for the first throw site a history met (the
// order of the checks follows the order in which the reference would raise).
int status_code(dp_ctx* ctx, int bits) {
  if (bits & DP_ST_DOMAIN_HI)  // src/MixedTransport.jl:45,155,196
    return fail(ctx, DP_ERR_DOMAIN,
                "Ancestor energy exceeds mixed tables; regenerate with larger K_max");
  if (bits & DP_ST_DOMAIN_LO)  // src/MixedTransport.jl:44
    return fail(ctx, DP_ERR_DOMAIN, "Below prepared mixed kernel domain");
  if (bits & DP_ST_ZERO_RATE)  // src/MixedTransport.jl:113
    return fail(ctx, DP_ERR_DOMAIN, "Cannot sample a zero-rate hard event");
  if (bits & DP_ST_BAD_WEIGHT)  // src/MixedTransport.jl:186
    return fail(ctx, DP_ERR_DOMAIN, "Invalid adjoint hard-event weight");
  if (bits & DP_ST_EVENT_CAP)  // src/MixedTransport.jl:193
    return fail(ctx, DP_ERR_STATE, "Mixed transport exceeded 100000 hard events; segment incomplete");
  if (bits & DP_ST_STEP_CAP)
    return fail(ctx, DP_ERR_STATE, "a history reached the transport step cap");
  if (bits & DP_ST_TABLE_WAIT)
    return fail(ctx, DP_ERR_STATE, "a table-staging wait exceeded its limit");
  if (bits & DP_ST_NO_PROGRESS)
    return fail(ctx, DP_ERR_STATE, "MC segment made no spatial progress");
  if (bits & DP_ST_BAD_MEDIUM)
    return fail(ctx, DP_ERR_ARG, "segment medium outside the media set");
  return DP_OK;
}

// Status bits of a finished run: the call's error code where the reference
// would have thrown (host synchronises).
int status_result(dp_ctx* ctx, const int* d_bits) {
  int bits = 0;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(&bits, d_bits, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  int rc = read_flag(ctx);
  if (rc) return rc;
  return status_code(ctx, bits);
}
int group_offsets(dp_ctx* ctx, const dp_los* los, const int64_t* given, long n, int64_t* off,
                  int64_t* coff, long expect) {
  los_offsets_kernel<<<1, 1024, 0, ctx->stream>>>(los, given, n, off, coff, expect, ctx->d_flag);
  ++ctx->launches;
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  return DP_OK;
}

long tally_jobs(long n, long total) { return n + total / kTallyChunk + 1; }
size_t tally_part_bytes() { return sizeof(TallyPart); }

int group_tally(dp_ctx* ctx, const double* contrib, const int32_t* status, const double* csda,
                const double* dcsda, const dp_los* los, const int32_t* valid, long n, long total,
                int sigma_n1, const int64_t* off, const int64_t* coff, void* part,
                dp_los_result* out, int* bits) {
  const long max_jobs = tally_jobs(n, total), warps_per_block = 8;
  TallyPart* tp = static_cast<TallyPart*>(part);
  timed_begin(ctx);
  los_chunk_kernel<<<int((max_jobs + warps_per_block - 1) / warps_per_block), 256, 0, ctx->stream>>>(
      contrib, status, off, coff, n, max_jobs, csda, dcsda, tp);
  los_tally_kernel<<<int((n + warps_per_block - 1) / warps_per_block), 256, 0, ctx->stream>>>(
      tp, off, coff, los, valid, n, csda ? 1 : 0, sigma_n1, out, bits);
  ++ctx->launches;  // the second of the pair (timed_begin counts the first)
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "mc_tally");
  return DP_OK;
}

}  // namespace mc
}  // namespace dp

namespace {

template <class R, int PHASE, int T, bool POR>
int launch_phase(dp_ctx* ctx, McParams& P, size_t smem, long max_blocks) {
  const int threads = T;
  DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(mc_kernel<R, PHASE, T, POR>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(mc_kernel<R, PHASE, T, POR>,
                                          cudaFuncAttributePreferredSharedMemoryCarveout,
                                          carveout_percent(ctx->device, smem)));
  int per_sm = 0, n_sm = 0;
  DP_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                         &per_sm, mc_kernel<R, PHASE, T, POR>, threads, smem));
  DP_CHECK_CUDA(ctx, cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
  if (per_sm < 1) return fail(ctx, DP_ERR_CUDA, "MC kernel does not fit on a multiprocessor");
  long blocks = std::min(long(per_sm) * n_sm, max_blocks);
  if (blocks < 1) blocks = 1;
  timed_begin(ctx);
  mc_kernel<R, PHASE, T, POR><<<int(blocks), threads, smem, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, sizeof(R) == 4 ? (PHASE ? "mc_mixed_hi" : "mc_mixed_lo")
                                : (PHASE ? "mc_fp64_hi" : "mc_fp64_lo"));
  return DP_OK;
}

// Both transport phases with CTAs of T threads (POR: the column has the
// porous layer, medium 2); P.queue must hold P.n handoff records and
// P.counter three zeroed words (set here).
template <class R, int T, bool POR>
int launch_mc_t(dp_ctx* ctx, McParams& P) {
  const int threads = T;
  P.coop_nel = std::max(P.info[0].nel, P.info[1].nel);
  if (POR) P.coop_nel = std::max(P.coop_nel, P.info[2].nel);
  const int warps = threads / 32;
  P.coop_kmax = 1;
  P.coop_kc = 0;
  P.sync = ctx->mc_sync[DP_KERNEL_MC][sizeof(R) == 4];
  P.coop_stride = KCfg<R>::coop ? coop_floats(P.coop_nel, 1) : 0;
  size_t coop_bytes = size_t(warps) * P.coop_stride * sizeof(float);
  size_t tables = size_t(POR ? 3 : 2) * P.lay.med_bytes;
  int dev_smem = 0;
  DP_CHECK_CUDA(ctx, cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
  P.staged = mc_smem_head<R>() + tables + coop_bytes <= size_t(dev_smem) &&
                     ctx->mc_stage[DP_KERNEL_MC][sizeof(R) == 4] == 0
                 ? 1
                 : 0;
  // the shared memory left after the tables (up to `cap` bytes in all)
  // batches DCS sums
  auto fit = [&](size_t cap) -> size_t {
    if (KCfg<R>::coop) {
      const size_t used = mc_smem_head<R>() + (P.staged ? tables : 0);
      P.coop_kmax = coop_kmax(cap - std::min(cap, used), warps, P.coop_nel);
      P.coop_stride = coop_floats(P.coop_nel, P.coop_kmax);
      coop_bytes = size_t(warps) * P.coop_stride * sizeof(float);
      P.coop_kc = cta_kc(warps * P.coop_stride, P.coop_nel, threads);
    }
    return mc_smem_head<R>() + (P.staged ? tables : 0) + coop_bytes;
  };
  size_t smem = fit(0);  // one event per warp: the least the kernel needs
  if (smem > size_t(dev_smem)) return fail(ctx, DP_ERR_ARG, "media too large for the MC kernel");
  // the DCS buffer fills the smallest carve-out step that holds it, the rest
  // of the SM's 256 KB is L1 for the spilled stack
  smem = fit(std::min(size_t(dev_smem), carveout_cap(smem)));
  long need = (P.n + threads - 1) / threads;
  long rec_blocks = std::min((P.n + 255) / 256, 152L * 32);
  DP_CHECK_CUDA(ctx, cudaMemsetAsync(P.counter, 0, 3 * sizeof(unsigned long long), ctx->stream));
  timed_begin(ctx);
  mc_init_kernel<R><<<int(rec_blocks), 256, 0, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "mc_init");
  if (P.order0) {
    timed_begin(ctx);
    DP_CHECK_CUDA(ctx, sched_order(ctx->stream, P.n, nullptr, KeyOf{P.key0}, P.sched, P.order0,
                                   &ctx->launches));
    --ctx->launches;  // timed_begin counted one of the three
    timed_end(ctx, "mc_order");
  }
  int rc = launch_phase<R, 0, T, POR>(ctx, P, smem, need);
  if (rc) return rc;
  if (P.order1) {
    // the queue that phase 0 filled, ordered by the histories' phase-1 cost
    using Q = typename std::conditional<POR, HandoffP<R>, Handoff<R>>::type;
    timed_begin(ctx);
    DP_CHECK_CUDA(ctx, sched_order(ctx->stream, P.n, P.counter + 2,
                                   QueueKeyOf<Q>{static_cast<const Q*>(P.queue), P.key1}, P.sched,
                                   P.order1, &ctx->launches));
    --ctx->launches;
    timed_end(ctx, "mc_order");
  }
  rc = launch_phase<R, 1, T, POR>(ctx, P, smem, need);
  if (rc) return rc;
  timed_begin(ctx);
  mc_finish_kernel<R><<<int(rec_blocks), 256, 0, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "mc_finish");
  return DP_OK;
}

// The porous-layer variant is compiled for the default CTA size only.
template <class R>
int launch_mc(dp_ctx* ctx, McParams& P) {
  if (P.porous) return launch_mc_t<R, KCfg<R>::threads, true>(ctx, P);
  return with_threads<R>(ctx->mc_threads[DP_KERNEL_MC][sizeof(R) == 4],
                         [&](auto t) { return launch_mc_t<R, decltype(t)::value, false>(ctx, P); });
}

int run(dp_ctx* ctx, McParams& P, int precision) {
  return precision == DP_PREC_MIXED ? launch_mc<float>(ctx, P) : launch_mc<double>(ctx, P);
}

McParams base_params(dp_ctx* ctx, const unsigned char* blob, const Layout& lay, const dp_mixture* rock,
                     const dp_mixture* air, const Consts& C, uint64_t seed) {
  McParams P{};
  P.blob = blob;
  P.lay = lay;
  P.info[0] = make_info(rock);
  P.info[1] = make_info(air);
  P.C = C;
  P.seed = seed;
  P.err_flag = ctx->d_flag;
  return P;
}

}  // namespace

int dp_mc_run_los(dp_ctx* ctx, const dp_physics* ph, dp_mixture* rock, const dp_mixture* air,
                  const dp_mc_config* cfg, long n_los, const dp_los* d_los, long total,
                  dp_los_result* d_out, double** contrib_out, int** status_or,
                  int compute_gradient, const dp_mixture* porous);

namespace {
// compiled CTA sizes of the persistent transport kernels (with_threads)
constexpr int kThreadsMixed[] = {1024, 768, 512};
constexpr int kThreadsFp64[] = {256};
bool shape_args(int family, int precision) {
  return (family == DP_KERNEL_MC || family == DP_KERNEL_DIR) &&
         (precision == DP_PREC_FP64 || precision == DP_PREC_MIXED);
}
}  // namespace

extern "C" {

int dp_mc_thread_choices(int precision, int* threads, int cap) {
  if (precision != DP_PREC_FP64 && precision != DP_PREC_MIXED) return DP_ERR_ARG;
  const int* list = precision == DP_PREC_MIXED ? kThreadsMixed : kThreadsFp64;
  const int n = precision == DP_PREC_MIXED ? 3 : 1;
  for (int i = 0; threads && i < std::min(n, cap); ++i) threads[i] = list[i];
  return n;
}

int dp_set_mc_threads(dp_ctx* ctx, int family, int precision, int threads) {
  if (!ctx || !shape_args(family, precision)) return fail(ctx, DP_ERR_ARG, "bad kernel family or precision");
  int list[8];
  const int n = dp_mc_thread_choices(precision, list, 8);
  if (threads != 0 && std::find(list, list + n, threads) == list + n)
    return fail(ctx, DP_ERR_ARG, "CTA size not compiled for this precision");
  ctx->mc_threads[family][precision] = threads;
  return DP_OK;
}

int dp_get_mc_threads(const dp_ctx* ctx, int family, int precision, int* threads) {
  if (!ctx || !threads || !shape_args(family, precision)) return DP_ERR_ARG;
  const int t = ctx->mc_threads[family][precision];
  *threads = t ? t : (precision == DP_PREC_MIXED ? kThreadsMixed[0] : kThreadsFp64[0]);
  return DP_OK;
}

int dp_set_mc_shape(dp_ctx* ctx, int family, int precision, const dp_mc_shape* shape) {
  if (!ctx || !shape || !shape_args(family, precision))
    return fail(ctx, DP_ERR_ARG, "bad kernel family, precision or shape");
  if (shape->staging != 0 && shape->staging != 1)
    return fail(ctx, DP_ERR_ARG, "staging is 0 (shared memory) or 1 (L1/L2)");
  if (shape->order != 0 && shape->order != 1)
    return fail(ctx, DP_ERR_ARG, "order is 0 (longest first) or 1 (index order)");
  if (shape->sync < 0 || shape->sync > 3)
    return fail(ctx, DP_ERR_ARG, "sync is a mask of the lockstep phases (0 to 3)");
  const int rc = dp_set_mc_threads(ctx, family, precision, shape->threads);
  if (rc) return rc;
  ctx->mc_stage[family][precision] = shape->staging;
  ctx->mc_order[family][precision] = shape->order;
  ctx->mc_sync[family][precision] = shape->sync;
  return DP_OK;
}

int dp_get_mc_shape(const dp_ctx* ctx, int family, int precision, dp_mc_shape* shape) {
  if (!ctx || !shape || !shape_args(family, precision)) return DP_ERR_ARG;
  dp_get_mc_threads(ctx, family, precision, &shape->threads);
  shape->staging = ctx->mc_stage[family][precision];
  shape->order = ctx->mc_order[family][precision];
  shape->sync = ctx->mc_sync[family][precision];
  return DP_OK;
}

int dp_autotune_shape(dp_ctx* ctx, int family, int precision, int (*run)(void*), void* user,
                      dp_mc_shape* best_out, dp_mc_shape* tried, double* ms, int cap,
                      int* n_tried) {
  if (!ctx || !run || !shape_args(family, precision))
    return fail(ctx, DP_ERR_ARG, "bad autotune arguments");
  dp_mc_shape saved{}, best{};
  dp_get_mc_shape(ctx, family, precision, &saved);
  best = saved;
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return fail(ctx, DP_ERR_CUDA, "event creation failed");
  }
  int rc = DP_OK, count = 0;
  float best_ms = -1.0f;
  // one candidate: run untimed (its code loads), then timed
  auto trial = [&](const dp_mc_shape& c) -> int {
    int r = dp_set_mc_shape(ctx, family, precision, &c);
    if (!r) r = run(user);
    if (!r && cudaEventRecord(a, ctx->stream) != cudaSuccess)
      r = fail(ctx, DP_ERR_CUDA, "event record failed");
    if (!r) r = run(user);
    if (!r && (cudaEventRecord(b, ctx->stream) != cudaSuccess ||
               cudaEventSynchronize(b) != cudaSuccess))
      r = fail(ctx, DP_ERR_CUDA, "event wait failed");
    if (r) return r;
    float t = 0.0f;
    cudaEventElapsedTime(&t, a, b);
    if (count < cap) {
      if (tried) tried[count] = c;
      if (ms) ms[count] = t;
    }
    ++count;
    if (best_ms < 0.0f || t < best_ms) {
      best_ms = t;
      best = c;
    }
    return DP_OK;
  };
  int list[8];
  const int nt = dp_mc_thread_choices(precision, list, 8);
  for (int i = 0; i < nt && !rc; ++i) {
    dp_mc_shape c = best;
    c.threads = list[i];
    rc = trial(c);
  }
  const dp_mc_shape after_threads = best;
  for (int st = 0; st < 2 && !rc; ++st)
    if (st != after_threads.staging) {
      dp_mc_shape c = after_threads;
      c.staging = st;
      rc = trial(c);
    }
  const dp_mc_shape after_stage = best;
  for (int od = 0; od < 2 && !rc; ++od)
    if (od != after_stage.order) {
      dp_mc_shape c = after_stage;
      c.order = od;
      rc = trial(c);
    }
  // the lockstep mask only changes the mixed-precision kernels
  const dp_mc_shape after_order = best;
  for (int sy = 0; sy < 4 && !rc && precision == DP_PREC_MIXED; ++sy)
    if (sy != after_order.sync) {
      dp_mc_shape c = after_order;
      c.sync = sy;
      rc = trial(c);
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (n_tried) *n_tried = count;
  if (rc) {
    dp_set_mc_shape(ctx, family, precision, &saved);
    return rc;
  }
  dp_set_mc_shape(ctx, family, precision, &best);
  if (best_out) *best_out = best;
  return DP_OK;
}

int dp_autotune(dp_ctx* ctx, int family, int precision, int (*run)(void*), void* user,
                int* best_threads, double* ms, int cap) {
  if (!ctx || !run || !shape_args(family, precision)) return fail(ctx, DP_ERR_ARG, "bad autotune arguments");
  int list[8];
  const int n = dp_mc_thread_choices(precision, list, 8);
  const int saved = ctx->mc_threads[family][precision];
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return fail(ctx, DP_ERR_CUDA, "event creation failed");
  }
  int best = 0, rc = DP_OK;
  float best_ms = 0.0f;
  for (int i = 0; i < n && !rc; ++i) {
    ctx->mc_threads[family][precision] = list[i];
    rc = run(user);  // untimed: first launch of this size loads its code
    if (rc) break;
    if (cudaEventRecord(a, ctx->stream) != cudaSuccess) rc = fail(ctx, DP_ERR_CUDA, "event record failed");
    if (!rc) rc = run(user);
    if (!rc && (cudaEventRecord(b, ctx->stream) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess))
      rc = fail(ctx, DP_ERR_CUDA, "event wait failed");
    if (rc) break;
    float t = 0.0f;
    cudaEventElapsedTime(&t, a, b);
    if (ms && i < cap) ms[i] = t;
    if (!best || t < best_ms) {
      best = list[i];
      best_ms = t;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) {
    ctx->mc_threads[family][precision] = saved;
    return rc;
  }
  ctx->mc_threads[family][precision] = best;
  if (best_threads) *best_threads = best;
  return DP_OK;
}

int dp_mixture_prepare(dp_ctx* ctx, const dp_physics* ph, int n, const int* mats,
                       const double* fracs, dp_mixture** out) {
  if (!ctx || !ph || !mats || !fracs || !out) return fail(ctx, DP_ERR_ARG, "null argument");
  dp_mixture* m = new dp_mixture;
  int rc = prepare(ctx, ph, n, mats, fracs, m);
  if (rc) {
    delete m;
    return rc;
  }
  *out = m;
  return DP_OK;
}

int dp_mixture_free(dp_mixture* m) {
  if (!m) return DP_OK;
  for (auto& b : m->blobs) cudaFree(b.dev);
  cudaGetLastError();  // a failed release must not surface at a later launch
  delete m;
  return DP_OK;
}

int dp_mixture_kernel(const dp_mixture* m, int col, double* out, int cap, int* n, double* onset) {
  if (!m || col < 0 || col >= K_NCOL) return DP_ERR_ARG;
  if (n) *n = m->nk;
  if (onset) *onset = m->onset;
  if (out && cap > 0)
    std::copy(m->kcols.begin() + size_t(col) * m->nk,
              m->kcols.begin() + size_t(col) * m->nk + std::min(cap, m->nk), out);
  return DP_OK;
}

int dp_mc_histories(dp_ctx* ctx, const dp_physics* ph, const dp_mixture* rock_c,
                    const dp_mixture* air, const dp_mc_config* cfg, long n, const double* E,
                    const double* q, const double* w, const double* thick, const double* dens,
                    const double* elev, const double* H, int geo_stride, uint64_t id0,
                    double* contrib, int32_t* status, int32_t* steps, double* efinal) {
  if (!ctx || !ph || !rock_c || !air) return fail(ctx, DP_ERR_ARG, "null argument");
  dp_mixture* rock = const_cast<dp_mixture*>(rock_c);
  Consts C;
  int rc = check_cfg(ctx, ph, cfg, &C);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!E || !q || !w || !thick || !dens || !elev || !H || !contrib)))
    return fail(ctx, DP_ERR_ARG, "bad history arrays");
  if (n == 0) return DP_OK;
  for (long i = 0; i < (geo_stride ? n : 1); ++i)
    if (!(dens[i] > 0.0) || !(thick[i] >= 0.0) || !(H[i] > 0.0))
      return fail(ctx, DP_ERR_ARG, "positive density and altitude, nonnegative thickness required");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  const unsigned char* blob;
  Layout lay;
  rc = get_blob(ctx, rock, air, cfg->precision, &blob, &lay);
  if (rc) return rc;
  long ng = geo_stride ? n : 1;
  size_t nb = size_t(n) * sizeof(double), gb = size_t(ng) * sizeof(double);
  Arena A;
  A.base = static_cast<char*>(scratch(
      ctx, 8 * nb + 4 * gb + size_t(n) * (8 + kRecBytes + kSchedBytes) + kSchedExtra + 4096, 0));
  A.cap = ctx->slot_bytes[0];
  double* dE = A.take<double>(n);
  double* dq = A.take<double>(n);
  double* dw = A.take<double>(n);
  double* dc = A.take<double>(n);
  double* dEf = A.take<double>(4 * n);
  double* dt = A.take<double>(ng);
  double* dd = A.take<double>(ng);
  double* de = A.take<double>(ng);
  double* dH = A.take<double>(ng);
  int32_t* ds = A.take<int32_t>(n);
  int32_t* dn = A.take<int32_t>(n);
  unsigned long long* ctr = A.take<unsigned long long>(3);
  Handoff<double>* queue = A.take<Handoff<double>>(n);
  StartRec<double>* srec = A.take<StartRec<double>>(n);
  EndRec<double>* erec = A.take<EndRec<double>>(n);
  if (!erec) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  cudaStream_t s = ctx->stream;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dE, E, nb, cudaMemcpyHostToDevice, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dq, q, nb, cudaMemcpyHostToDevice, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dw, w, nb, cudaMemcpyHostToDevice, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dt, thick, gb, cudaMemcpyHostToDevice, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dd, dens, gb, cudaMemcpyHostToDevice, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(de, elev, gb, cudaMemcpyHostToDevice, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dH, H, gb, cudaMemcpyHostToDevice, s));
  McParams P = base_params(ctx, blob, lay, rock, air, C, cfg->seed);
  P.source = 0;
  P.n = n;
  P.id0 = id0;
  P.E = dE;
  P.q = dq;
  P.w = dw;
  P.thick = dt;
  P.dens = dd;
  P.elev = de;
  P.H = dH;
  P.geo_stride = geo_stride ? 1 : 0;
  P.contrib = dc;
  P.status = ds;
  P.steps = dn;
  P.efinal = dEf;
  P.counter = ctr;
  P.queue = queue;
  P.start = srec;
  P.end = erec;
  take_sched(ctx, cfg->precision, n, A, P);
  rc = run(ctx, P, cfg->precision);
  if (rc) return rc;
  std::vector<int32_t> st_h;
  if (!status) {
    st_h.resize(n);
    status = st_h.data();
  }
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(contrib, dc, nb, cudaMemcpyDeviceToHost, s));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(status, ds, size_t(n) * 4, cudaMemcpyDeviceToHost, s));
  if (steps) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(steps, dn, size_t(n) * 4, cudaMemcpyDeviceToHost, s));
  if (efinal) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(efinal, dEf, 4 * nb, cudaMemcpyDeviceToHost, s));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  rc = read_flag(ctx);
  if (rc) return rc;
  int bits = 0;
  for (long i = 0; i < n; ++i) bits |= status[i];
  return status_code(ctx, bits);
}

int dp_mc_los_layers_dev(dp_ctx* ctx, const dp_physics* ph, const dp_mixture* rock_c,
                         const dp_mixture* porous, const dp_mixture* air,
                         const dp_mc_config* cfg, long n_los, const dp_los* los, long total,
                         int compute_gradient, dp_los_result* out) {
  if (!ctx || !ph || !rock_c || !air || !los || !out || n_los <= 0 || total < 0)
    return fail(ctx, DP_ERR_ARG, "bad arguments");
  if (porous && compute_gradient)
    return fail(ctx, DP_ERR_ARG, "the CSDA gradient has no porous layer");
  double* contrib = nullptr;
  int* bits = nullptr;
  int rc = dp_mc_run_los(ctx, ph, const_cast<dp_mixture*>(rock_c), air, cfg, n_los, los, total, out,
                         &contrib, &bits, compute_gradient, porous);
  if (rc) return rc;
  if (ctx->blocking) return status_result(ctx, bits);
  return DP_OK;
}

int dp_mc_los_dev(dp_ctx* ctx, const dp_physics* ph, const dp_mixture* rock_c,
                  const dp_mixture* air, const dp_mc_config* cfg, long n_los, const dp_los* los,
                  long total, int compute_gradient, dp_los_result* out) {
  return dp_mc_los_layers_dev(ctx, ph, rock_c, nullptr, air, cfg, n_los, los, total,
                              compute_gradient, out);
}

int dp_mc_los(dp_ctx* ctx, const dp_physics* ph, const dp_mixture* rock, const dp_mixture* air,
              const dp_mc_config* cfg, long n_los, const dp_los* los, int compute_gradient,
              dp_los_result* out) {
  return dp_mc_los_layers(ctx, ph, rock, nullptr, air, cfg, n_los, los, compute_gradient, out);
}

int dp_mc_los_layers(dp_ctx* ctx, const dp_physics* ph, const dp_mixture* rock,
                     const dp_mixture* porous, const dp_mixture* air, const dp_mc_config* cfg,
                     long n_los, const dp_los* los, int compute_gradient, dp_los_result* out) {
  if (!ctx || !los || !out || n_los <= 0) return fail(ctx, DP_ERR_ARG, "bad arguments");
  if (porous && compute_gradient)
    return fail(ctx, DP_ERR_ARG, "the CSDA gradient has no porous layer");
  long total = 0;
  for (long l = 0; l < n_los; ++l) {
    const dp_los& L = los[l];
    if (L.n_samples < 0) return fail(ctx, DP_ERR_ARG, "negative n_samples");
    if (!(L.energy_min > 0.0)) return fail(ctx, DP_ERR_ARG, "energy_min must be positive");
    // transport_mixed_step needs a positive density (src/MixedTransport.jl:146)
    if (!(L.density > 0.0) || !(L.thickness >= 0.0))
      return fail(ctx, DP_ERR_ARG, "positive density and nonnegative thickness required");
    if (porous && L.porous_thickness > 0.0 && !(L.porous_density > 0.0))
      return fail(ctx, DP_ERR_ARG, "a porous layer needs a positive density");
    total += L.n_samples;
  }
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  Arena A;
  size_t lb = size_t(n_los) * sizeof(dp_los), ob = size_t(n_los) * sizeof(dp_los_result);
  A.base = static_cast<char*>(scratch(ctx, lb + ob + 1024, 2));
  A.cap = ctx->slot_bytes[2];
  dp_los* dl = A.take<dp_los>(n_los);
  dp_los_result* dr = A.take<dp_los_result>(n_los);
  if (!dr) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dl, los, lb, cudaMemcpyHostToDevice, ctx->stream));
  if (compute_gradient)
    for (long l = 0; l < n_los; ++l)
      if (los[l].thickness_max > los[l].thickness || los[l].density_max > los[l].density ||
          los[l].elevation_max > los[l].elevation)
        return fail(ctx, DP_ERR_ARG, "the CSDA gradient needs fixed line-of-sight geometry");
  double* contrib = nullptr;
  int* bits = nullptr;
  int rc = dp_mc_run_los(ctx, ph, const_cast<dp_mixture*>(rock), air, cfg, n_los, dl, total, dr,
                         &contrib, &bits, compute_gradient, porous);
  if (rc) return rc;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(out, dr, ob, cudaMemcpyDeviceToHost, ctx->stream));
  return status_result(ctx, bits);
}

}  // extern "C"

// Enqueues one batched run over n_los lines of sight (device records) and
// the per-line-of-sight tallies; *contrib_out receives the per-history
// contributions (scratch slot 0, valid until the next call on ctx).
int dp_mc_run_los(dp_ctx* ctx, const dp_physics* ph, dp_mixture* rock, const dp_mixture* air,
                  const dp_mc_config* cfg, long n_los, const dp_los* d_los, long total,
                  dp_los_result* d_out, double** contrib_out, int** status_or,
                  int compute_gradient, const dp_mixture* porous) {
  Consts C;
  double thr64;
  int rc = check_cfg(ctx, ph, cfg, &C, &thr64);
  if (rc) return rc;
  if (compute_gradient && (rock->nm != 1 || air->nm != 1))
    return fail(ctx, DP_ERR_ARG, "the CSDA gradient needs single-material rock and air");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  const unsigned char* blob;
  Layout lay;
  rc = get_blob(ctx, rock, air, cfg->precision, &blob, &lay, porous);
  if (rc) return rc;
  long nt = total > 0 ? total : 1;
  Arena A;
  A.base = static_cast<char*>(scratch(
      ctx, size_t(nt) * (12 + 16 + kRecBytes + kSchedBytes) + size_t(n_los + 1) * 16 +
               size_t(n_los + nt / kTallyChunk + 1) * sizeof(TallyPart) + kSchedExtra + 4096, 0));
  A.cap = ctx->slot_bytes[0];
  double* dc = A.take<double>(nt);
  int32_t* ds = A.take<int32_t>(nt);
  int64_t* off = A.take<int64_t>(n_los + 1);
  int64_t* coff = A.take<int64_t>(n_los + 1);
  TallyPart* tpart = A.take<TallyPart>(tally_jobs(n_los, nt));
  unsigned long long* ctr = A.take<unsigned long long>(3);
  HandoffP<double>* queue = A.take<HandoffP<double>>(nt);
  StartRec<double>* srec = A.take<StartRec<double>>(nt);
  EndRec<double>* erec = A.take<EndRec<double>>(nt);
  PorousRec<double>* prec = porous ? A.take<PorousRec<double>>(nt) : nullptr;
  double* cc = compute_gradient ? A.take<double>(nt) : nullptr;
  double* cd = compute_gradient ? A.take<double>(nt) : nullptr;
  int* bits = A.take<int>(1);
  if (!bits) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  DP_CHECK_CUDA(ctx, cudaMemsetAsync(bits, 0, sizeof(int), ctx->stream));
  rc = group_offsets(ctx, d_los, nullptr, n_los, off, coff, total);
  if (rc) return rc;
  if (total > 0) {
    McParams P = base_params(ctx, blob, lay, rock, air, C, cfg->seed);
    P.source = 1;
    P.n = total;
    P.los = d_los;
    P.los_off = off;
    P.n_los = n_los;
    P.contrib = dc;
    P.status = ds;
    P.counter = ctr;
    P.queue = queue;
    P.start = srec;
    P.end = erec;
    if (porous) {
      P.porous = 1;
      P.info[2] = make_info(porous);
      P.porous_rec = prec;
    }
    take_sched(ctx, cfg->precision, total, A, P);
    rc = run(ctx, P, cfg->precision);
    if (rc) return rc;
    if (compute_gradient) {
      // deterministic CSDA surrogate over the same samples (src/Geometry.jl:933-945)
      rc = csda_los(ctx, ph, rock->mats[0], air->mats[0], thr64,
                    cfg->energy_threshold_low > 0.0 ? cfg->energy_threshold_low : 100.0,
                    cfg->seed, d_los, off, n_los, total, cc, cd, cfg->precision);
      if (rc) return rc;
    }
  }
  rc = group_tally(ctx, dc, ds, total > 0 ? cc : nullptr, cd, d_los, nullptr, n_los, total, 0, off,
                   coff, tpart, d_out, bits);
  if (rc) return rc;
  if (contrib_out) *contrib_out = dc;
  if (status_or) *status_or = bits;
  return DP_OK;
}

namespace dp {
int mc_backward_stochastic(dp_ctx* ctx, const dp_physics* ph, const dp_mc_params* p, int rock,
                           int air, double threshold, dp_los_result* res) {
  dp_mixture rm, am, pm;
  const double one = 1.0;
  const bool porous = p->porous_material >= 0 && p->porous_thickness > 0.0;
  int rc = prepare(ctx, ph, 1, &rock, &one, &rm);
  if (!rc) rc = prepare(ctx, ph, 1, &air, &one, &am);
  if (!rc && porous) rc = prepare(ctx, ph, 1, &p->porous_material, &one, &pm);
  if (rc) return rc;
  dp_mc_config cfg{};
  cfg.straggling = p->straggling;
  cfg.scattering = p->scattering;
  cfg.energy_threshold_low = p->energy_threshold_low;
  cfg.source_energy_max = threshold;
  cfg.seed = p->seed;
  cfg.precision = p->precision;
  dp_los L{};
  L.thickness = p->rock_thickness;
  L.density = p->rock_density;
  L.elevation = p->elevation;
  L.primary_altitude = p->primary_altitude > 0.0 ? p->primary_altitude : 3e4;
  L.energy_min = p->energy_min;
  L.energy_max = p->energy_max > p->energy_min ? p->energy_max : p->energy_min;
  L.n_samples = p->n_samples;
  if (porous) {
    L.porous_thickness = p->porous_thickness;
    L.porous_density = p->porous_density;
  }
  Arena A;
  A.base = static_cast<char*>(scratch(ctx, sizeof(dp_los) + sizeof(dp_los_result) + 1024, 2));
  A.cap = ctx->slot_bytes[2];
  dp_los* dl = A.take<dp_los>(1);
  dp_los_result* dr = A.take<dp_los_result>(1);
  if (!dr) rc = fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  int* bits = nullptr;
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(dl, &L, sizeof(L), cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "cudaMemcpyAsync");
  }
  if (!rc)
    rc = dp_mc_run_los(ctx, ph, &rm, &am, &cfg, 1, dl, p->n_samples, dr, nullptr, &bits, 0,
                       porous ? &pm : nullptr);
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(res, dr, sizeof(*res), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "cudaMemcpyAsync");
  }
  if (!rc) rc = status_result(ctx, bits);
  cudaStreamSynchronize(ctx->stream);
  for (auto& b : rm.blobs) cudaFree(b.dev);
  return rc;
}
}  // namespace dp

// mc_device.cuh -- device side of the stochastic backward Monte Carlo: one
// thread per history, templated on the transport arithmetic R (double: the
// reference's FP64 operations; float: the mixed-precision form, where
// positions, event kinematics, DCS and the flux stay FP64).
//
// Restates src/Geometry.jl:148-357 (straggled step), :424-457 (CSDA step),
// :461-476 (step limit), :534-672 (dual-mode loop), :694-757 (acceptance),
// src/MixedTransport.jl:43-200 (MIXED kernel lookups, adjoint hard events,
// mixed step) and src/Straggling.jl (fluctuations, EHS, angles, rotations).
// Random numbers: Philox4x32-10 keyed by the seed with counter (history id,
// block); block 0 holds the energy/charge draws, blocks 1-2 the drawn
// geometry, transport draws start at block 3.
#pragma once
#include <math_constants.h>

#include <type_traits>

#include "common.cuh"
#include "dcs.cuh"

namespace dp {
namespace mc {

constexpr int kMaxMix = 4;   // materials in one mixture medium
constexpr int kMaxEl = 32;   // elements in one medium
constexpr int kElStride = 5; // Z, A, I, fraction, nuclear RMS radius (m)
constexpr double kEhsPathMax = 1e9;
constexpr uint32_t kTransportBlock = 3;

enum : int {
  ST_STEP_CAP = DP_ST_STEP_CAP,
  ST_OUTER_CAP = DP_ST_OUTER_CAP,
  ST_EVENT_CAP = DP_ST_EVENT_CAP,
  ST_DOMAIN_HI = DP_ST_DOMAIN_HI,
  ST_DOMAIN_LO = DP_ST_DOMAIN_LO,
  ST_ZERO_RATE = DP_ST_ZERO_RATE,
  ST_BAD_WEIGHT = DP_ST_BAD_WEIGHT,
  ST_TABLE = DP_ST_TABLE_WAIT,
  ST_NO_PROGRESS = DP_ST_NO_PROGRESS,
  ST_BAD_MEDIUM = DP_ST_BAD_MEDIUM,
  ST_FATAL = ST_STEP_CAP | ST_EVENT_CAP | ST_DOMAIN_HI | ST_DOMAIN_LO | ST_ZERO_RATE |
             ST_BAD_WEIGHT | ST_TABLE | ST_NO_PROGRESS | ST_BAD_MEDIUM,
};

// Packed medium (one blob per medium and precision, the same layout for
// every medium of a launch): kMaxEl elements of kElStride doubles, then the
// physics-grid columns (stride ld), then the MIXED kernel columns (stride ldk).
// Physics-grid columns: MC_E ... MC_FSPIN, then `slots` transport-path columns
// (one per mixture material) and `slots` elastic-path columns.
enum MedCol { MC_E = 0, MC_LE, MC_CS, MC_CR, MC_MS, MC_MR, MC_STRAG, MC_MU0, MC_FSPIN, MC_LB1 };
// MIXED kernel columns (src/MixedTransport.jl:15-29).
enum KerCol { K_E = 0, K_S, K_SIG, K_R, K_H, K_T, K_NCOL };

struct Layout {
  uint32_t med_bytes;  // bytes of one medium (16-byte multiple)
  uint32_t o_phys;     // byte offset of the physics columns
  uint32_t o_ker;      // byte offset of the kernel columns
  int ld, ldk;         // column strides (elements)
  int n, nk, slots, uniform;
  double lE0, inv_dlE;
  int kuniform;        // MIXED kernel energies: the uniform log grid refined 8-fold
  double kinv_dlE;     // 1 / log step of the kernel energies
  uint32_t o_idx;      // byte offset of the inverse-lookup index tables (int16)
  int nbp, nbk;        // index bins of the physics and kernel columns
  uint32_t o_elf;      // byte offset of the FP32 element table (kElfStride floats each)
};
// FP32 element table for the cooperative DCS sums and the FP32 polar angles:
// Z, A, I, fraction, N_A / (A 1e-3) (per-mass scale), nuclear RMS radius (m).
constexpr int kElfStride = 8;

// Inverse lookups (energy from a range or hazard value) start from an index
// table over log-uniform bins of the column's values instead of a bisection:
// entry b holds the last node at or below the bin's lower edge; the search
// then walks up (a few nodes).  Columns: 0 CSDA range, 1 restricted range
// (physics grid), 2 kernel range, 3 kernel hazard.  Per column the bin
// origin and inverse width (two doubles) follow the elements.
enum IdxCol { I_CR = 0, I_MR, I_KR, I_KH, I_NCOL };
constexpr int kIdxBinsPhys = 256, kIdxBinsKer = 1024;
struct MedInfo {
  int nm, nel;
  double frac[kMaxMix];
  double ZoA, onset;
};

template <class R>
struct Med {
  const R* p;
  const R* kp;
  const double* el;
  const float* elf;
  const int16_t* idx;
  int ld, ldk, n, nk, nm, nel, slots, uniform, kuniform;
  R frac[kMaxMix];
  R ZoA, onset, lE0, inv_dlE, kinv_dlE;
  __device__ __forceinline__ const R* col(int k) const { return p + k * ld; }
  __device__ __forceinline__ const R* kcol(int j) const { return kp + j * ldk; }
  __device__ __forceinline__ int lbe(int j) const { return MC_LB1 + slots + j; }
};

template <class R>
__device__ __forceinline__ Med<R> make_med(const unsigned char* base, const Layout& L,
                                           const MedInfo& I) {
  Med<R> m;
  m.p = reinterpret_cast<const R*>(base + L.o_phys);
  m.kp = reinterpret_cast<const R*>(base + L.o_ker);
  m.el = reinterpret_cast<const double*>(base);
  m.elf = reinterpret_cast<const float*>(base + L.o_elf);
  m.idx = reinterpret_cast<const int16_t*>(base + L.o_idx);
  m.ld = L.ld;
  m.ldk = L.ldk;
  m.n = L.n;
  m.nk = L.nk;
  m.slots = L.slots;
  m.uniform = L.uniform;
  m.lE0 = R(L.lE0);
  m.inv_dlE = R(L.inv_dlE);
  m.kuniform = L.kuniform;
  m.kinv_dlE = R(L.kinv_dlE);
  m.nm = I.nm;
  m.nel = I.nel;
#pragma unroll
  for (int j = 0; j < kMaxMix; ++j) m.frac[j] = R(I.frac[j]);
  m.ZoA = R(I.ZoA);
  m.onset = R(I.onset);
  return m;
}

// Run constants shared by every history of a launch.
struct Consts {
  double mass, ctau, cutoff, elastic_ratio;
  double thr_low, thr;  // mode switch and source ceiling (GeV)
  float thr_low_f, thr_f;  // the same in FP32 (exact for the FP32 transport)
  float mass_f, ctau_f, elastic_ratio_f;
  float cutoff_f, lcut_f;  // cutoff and -log(cutoff) in FP32
  int straggling, scattering;
  // loop caps and the table-staging wait limit of the launch
  int step_cap, event_cap, wait_iters;
  // physics constants in the transport precision
  template <class R> __device__ __forceinline__ R mass_r() const {
    return sizeof(R) == 8 ? R(mass) : R(mass_f);
  }
  template <class R> __device__ __forceinline__ R ctau_r() const {
    return sizeof(R) == 8 ? R(ctau) : R(ctau_f);
  }
  template <class R> __device__ __forceinline__ R eratio_r() const {
    return sizeof(R) == 8 ? R(elastic_ratio) : R(elastic_ratio_f);
  }
};

// ------------------------------------------------------------ random stream
struct Stream {
  uint32_t k0, k1, c0, c1, block, w0, w1, w2, w3;
  int used;
  __device__ __forceinline__ void init(uint64_t seed, uint64_t id) {
    k0 = uint32_t(seed);
    k1 = uint32_t(seed >> 32);
    c0 = uint32_t(id);
    c1 = uint32_t(id >> 32);
    block = kTransportBlock;
    used = 2;
  }
  __device__ __forceinline__ void next(uint32_t& a, uint32_t& b);
};
// One Philox block for the stream (kept out of line: every draw site would
// otherwise carry the ten unrolled rounds).
static __device__ __noinline__ U4 philox_block(uint32_t c0, uint32_t c1, uint32_t block, uint32_t k0,
                                        uint32_t k1) {
  return philox(U4{c0, c1, block, 0u}, k0, k1);
}
__device__ __forceinline__ void Stream::next(uint32_t& a, uint32_t& b) {
  if (used >= 2) {
    U4 r = philox_block(c0, c1, block, k0, k1);
    ++block;
    w0 = r.x;
    w1 = r.y;
    w2 = r.z;
    w3 = r.w;
    used = 0;
  }
  a = used == 0 ? w0 : w2;
  b = used == 0 ? w1 : w3;
  ++used;
}
template <class R> __device__ __forceinline__ R uni(Stream& g);
template <> __device__ __forceinline__ double uni<double>(Stream& g) {
  uint32_t a, b;
  g.next(a, b);
  return u01(a, b);
}
// The leading 24 bits of the same draw (it differs from the double by < 2^-24).
// FP32: 24 bits of the draw, in (0, 1).  A 24-bit uniform of exactly 0
// (probability 2^-24, against 2^-53 in FP64) would place a hard event at zero
// grammage, a step of no length that the fixed-path loop rejects
// (src/Tomography.jl:916): the lowest bin maps to 2^-25 instead.
template <> __device__ __forceinline__ float uni<float>(Stream& g) {
  uint32_t a, b;
  g.next(a, b);
  return fmaxf(float(a >> 8) * 0x1p-24f, 0x1p-25f);
}
__device__ __forceinline__ double uni_d(Stream& g) {
  uint32_t a, b;
  g.next(a, b);
  return u01(a, b);
}
template <class R> __device__ __forceinline__ R expo(Stream& g) { return -log1p(-uni<R>(g)); }

template <class R> __device__ __forceinline__ R ulp_up(R x);
template <> __device__ __forceinline__ double ulp_up<double>(double x) {
  return nextafter(x, CUDART_INF) - x;
}
template <> __device__ __forceinline__ float ulp_up<float>(float x) {
  return nextafterf(x, CUDART_INF_F) - x;
}

// ------------------------------------------------------------ physics grid
template <class R>
__device__ __forceinline__ int bisect_r(const R* xs, int n, R x) {
  int lo = 0, hi = n - 1;
  while (lo < hi - 1) {
    int mid = (lo + hi) >> 1;
    if (x < xs[mid]) hi = mid; else lo = mid;
  }
  return lo;
}

// Interval of x on the physics grid (src/Physics.jl:660-687): clamped ends,
// else linear in log E.  One location serves every column at that energy.
template <class R>
struct Loc {
  int i, edge;
  R t;
};
template <class R>
__device__ __forceinline__ Loc<R> locate(const Med<R>& m, R x) {
  Loc<R> L{0, 0, R(0)};
  const R* E = m.col(MC_E);
  if (x <= E[0]) {
    L.edge = -1;
    return L;
  }
  if (x >= E[m.n - 1]) {
    L.edge = 1;
    return L;
  }
  const R* lE = m.col(MC_LE);
  R lx = log(x);
  int i;
  if (m.uniform) {
    R f = floor((lx - m.lE0) * m.inv_dlE);
    i = !(f >= R(0)) ? 0 : (f > R(m.n - 2) ? m.n - 2 : int(f));
    while (i > 0 && lx < lE[i]) --i;
    while (i < m.n - 2 && !(lx < lE[i + 1])) ++i;
  } else {
    i = bisect_r(lE, m.n, lx);
  }
  L.i = i;
  L.t = (lx - lE[i]) / (lE[i + 1] - lE[i]);
  return L;
}
template <class R>
__device__ __forceinline__ R at(const Med<R>& m, const Loc<R>& L, int col) {
  const R* y = m.col(col);
  if (L.edge < 0) return y[0];
  if (L.edge > 0) return y[m.n - 1];
  return y[L.i] + L.t * (y[L.i + 1] - y[L.i]);
}
// Starting node of an inverse lookup of x in index column `which`.
template <class R>
__device__ __forceinline__ int index_guess(const Med<R>& m, int which, R x) {
  const R* prm = reinterpret_cast<const R*>(m.el + kMaxEl * kElStride) + 2 * which;
  const int nb = which < I_KR ? kIdxBinsPhys : kIdxBinsKer;
  const int16_t* idx = m.idx + (which < I_KR ? which * kIdxBinsPhys
                                             : 2 * kIdxBinsPhys + (which - I_KR) * kIdxBinsKer);
  if (!(x > R(0))) return 0;
  R f = (log(x) - prm[0]) * prm[1];
  int b = !(f >= R(0)) ? 0 : (f >= R(nb) ? nb - 1 : int(f));
  return idx[b];
}
// Largest i in [0, n-2] with xs[i] <= x, walking from a guess (equals the
// bisection for x inside (xs[0], xs[n-1])).
template <class R>
__device__ __forceinline__ int walk_from(const R* xs, int n, R x, int i) {
  i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
  while (i > 0 && x < xs[i]) --i;
  while (i < n - 2 && !(x < xs[i + 1])) ++i;
  return i;
}

// Inverse of a range column (src/Physics.jl:833-867).
template <class R>
__device__ __forceinline__ R inv_range(const Med<R>& m, int col, R X) {
  const R* Rc = m.col(col);
  int n = m.n;
  if (X <= Rc[0]) return m.col(MC_E)[0];
  if (X >= Rc[n - 1]) return m.col(MC_E)[n - 1];
  int i = walk_from(Rc, n, X, index_guess(m, col == MC_CR ? I_CR : I_MR, X));
  const R* lE = m.col(MC_LE);
  R t = (X - Rc[i]) / (Rc[i + 1] - Rc[i]);
  return exp(lE[i] + t * (lE[i + 1] - lE[i]));
}

// property_transport_path of a material or a mixture (harmonic, src/Physics.jl:912, :1220).
template <class R>
__device__ __forceinline__ R transport_path(const Med<R>& m, const Loc<R>& L) {
  if (m.nm == 1) return at(m, L, MC_LB1);
  R inv = R(0);
  for (int j = 0; j < m.nm; ++j) {
    R lp = at(m, L, MC_LB1 + j);
    if (lp > R(0)) inv += m.frac[j] / lp;
  }
  return inv > R(0) ? R(1) / inv : R(1e9);
}
// compute_ehs_mean_free_path (src/Straggling.jl:330-360, :1025-1038).
template <class R>
__device__ __forceinline__ R ehs_single(const Med<R>& m, int j, R K, const Loc<R>& L, R mass,
                                        R elastic_ratio) {
  if (K < R(1e-3)) return R(kEhsPathMax);
  R Lb = at(m, L, m.lbe(j));
  R p2 = K * (K + R(2) * mass);
  if (Lb > R(0) && Lb < R(kEhsPathMax) * p2) return Lb / p2;
  R tp = at(m, L, MC_LB1 + j);
  if (tp > R(0)) return fmin(tp / elastic_ratio, R(kEhsPathMax));
  return R(kEhsPathMax);
}
template <class R>
__device__ __forceinline__ R ehs_path(const Med<R>& m, R K, R mass, R elastic_ratio) {
  Loc<R> L = locate(m, K);
  if (m.nm == 1) return ehs_single(m, 0, K, L, mass, elastic_ratio);
  R inv = R(0);
  for (int j = 0; j < m.nm; ++j) {
    R lp = ehs_single(m, j, K, L, mass, elastic_ratio);
    if (lp > R(0) && lp < R(kEhsPathMax)) inv += m.frac[j] / lp;
  }
  return inv > R(0) ? R(1) / inv : R(kEhsPathMax);
}

// ------------------------------------------------------------ MIXED kernel
// searchsortedlast lookup (src/MixedTransport.jl:43-49); values outside the
// table set the domain bits (the reference throws DomainError there).
template <class R>
struct KLoc {
  int i, edge;
  R f;
};
template <class R>
__device__ __forceinline__ KLoc<R> klocate(const R* xs, int n, R x, int* status) {
  KLoc<R> L{0, 0, R(0)};
  if (x < xs[0]) {
    *status |= ST_DOMAIN_LO;
    L.edge = -1;
    return L;
  }
  if (x > xs[n - 1]) {
    *status |= ST_DOMAIN_HI;
    L.edge = 1;
    return L;
  }
  int lo = 0, hi = n;  // first index with xs[idx] > x
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (xs[mid] <= x) lo = mid + 1; else hi = mid;
  }
  int i = (lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo)) - 1;
  R d = xs[i + 1] - xs[i];
  L.i = i;
  L.f = d == R(0) ? R(0) : (x - xs[i]) / d;
  return L;
}
template <class R>
__device__ __forceinline__ R kat(const R* ys, int n, const KLoc<R>& L) {
  if (L.edge < 0) return ys[0];
  if (L.edge > 0) return ys[n - 1];
  return ys[L.i] + L.f * (ys[L.i + 1] - ys[L.i]);
}
// The same location on the kernel's energy axis: on a uniform log grid an
// O(1) guess corrected to the searchsortedlast interval.
template <class R>
__device__ __forceinline__ KLoc<R> klocate_e(const Med<R>& m, R x, int* status) {
  const R* xs = m.kcol(K_E);
  const int n = m.nk;
  if (!m.kuniform || !(x == x)) return klocate(xs, n, x, status);
  KLoc<R> L{0, 0, R(0)};
  if (x < xs[0]) {
    *status |= ST_DOMAIN_LO;
    L.edge = -1;
    return L;
  }
  if (x > xs[n - 1]) {
    *status |= ST_DOMAIN_HI;
    L.edge = 1;
    return L;
  }
  R f = floor((log(x) - m.lE0) * m.kinv_dlE);
  int i = !(f >= R(0)) ? 0 : (f > R(n - 2) ? n - 2 : int(f));
  while (i > 0 && x < xs[i]) --i;
  while (i < n - 2 && !(x < xs[i + 1])) ++i;
  R d = xs[i + 1] - xs[i];
  L.i = i;
  L.f = d == R(0) ? R(0) : (x - xs[i]) / d;
  return L;
}
// searchsortedlast location on the kernel's range or hazard axis from its
// index table.
template <class R>
__device__ __forceinline__ KLoc<R> klocate_idx(const Med<R>& m, int xcol, R x, int* status) {
  const R* xs = m.kcol(xcol);
  const int n = m.nk;
  KLoc<R> L{0, 0, R(0)};
  if (x < xs[0]) {
    *status |= ST_DOMAIN_LO;
    L.edge = -1;
    return L;
  }
  if (x > xs[n - 1]) {
    *status |= ST_DOMAIN_HI;
    L.edge = 1;
    return L;
  }
  if (!(x == x)) return klocate(xs, n, x, status);
  int i = walk_from(xs, n, x, index_guess(m, xcol == K_R ? I_KR : I_KH, x));
  R d = xs[i + 1] - xs[i];
  L.i = i;
  L.f = d == R(0) ? R(0) : (x - xs[i]) / d;
  return L;
}
template <class R>
__device__ __forceinline__ R klookup(const Med<R>& m, int xcol, int ycol, R x, int* status) {
  if (xcol == K_E) return kat(m.kcol(ycol), m.nk, klocate_e(m, x, status));
  if (xcol == K_R || xcol == K_H) return kat(m.kcol(ycol), m.nk, klocate_idx(m, xcol, x, status));
  return kat(m.kcol(ycol), m.nk, klocate(m.kcol(xcol), m.nk, x, status));
}

// Sum over elements and processes of f * dsigma/dq (src/MixedTransport.jl:99-106)
// by one thread in FP64 (the FP64 transport), in the reference's order.
static __device__ __noinline__ double del_total(const double* el, int nel, double mass, double anc,
                                         double q) {
  double total = 0.0;
  for (int e = 0; e < nel; ++e) {
    const double* x = el + kElStride * e;
    double f = x[3] * kAvogadro / (x[1] * 0.001) * anc;
    total += f * dcs_brems(x[0], x[1], mass, anc, q);
    total += f * dcs_pair(x[0], x[1], mass, anc, q);
    total += f * dcs_photo(x[0], x[1], mass, anc, q);
    total += f * dcs_ionisation(x[0], x[2], mass, anc, q);
  }
  return total;
}
// Index of the component whose running sum first exceeds u (the process and
// element pick of src/MixedTransport.jl:131-140).
static __device__ __noinline__ int del_pick(const double* el, int nel, double mass, double anc, double q,
                                     double u) {
  int last = 4 * nel - 1;
  for (int i = 0; i <= last; ++i) {
    const double* x = el + kElStride * (i / 4);
    double f = x[3] * kAvogadro / (x[1] * 0.001) * anc;
    int p = i % 4;
    double v = p == 0 ? dcs_brems(x[0], x[1], mass, anc, q)
               : p == 1 ? dcs_pair(x[0], x[1], mass, anc, q)
               : p == 2 ? dcs_photo(x[0], x[1], mass, anc, q)
                        : dcs_ionisation(x[0], x[2], mass, anc, q);
    u -= f * v;
    if (u <= 0.0) return i;
  }
  return last;
}

// Terms of one hard-event DCS sum spread over a warp: per element one
// bremsstrahlung, 12 pair-asymmetry and 9 photonuclear quadrature points and
// one ionisation term.
constexpr int kItemsPerElement = 23;

// Per-warp buffer of the batched DCS sums, for up to kmax events of a medium
// with nel elements: the items (kItemsPerElement x nel floats per event), the
// components (4 x nel per event) and the totals (one per event), then, on a
// 16-byte boundary, the events' ancestor energies and energy transfers.
// coop_floats is its size in floats.
__host__ __device__ inline int coop_head(int nel, int kmax) {
  return (kmax * ((kItemsPerElement + 4) * nel + 1) + 3) / 4 * 4;
}
__host__ __device__ inline int coop_floats(int nel, int kmax) {
  return coop_head(nel, kmax) + 4 * kmax;
}

// The items of one event's DCS sum in FP32 (element table row x, mass fm,
// ancestor energy fk, transfer fq): pair-production asymmetry point p (items
// 1..12 of an element), photonuclear point p (items 13..21), and
// bremsstrahlung (t = 0, item 0) or ionisation (t = 1, item 22).  Shared by
// the warp and the CTA forms of the batched sums.
__device__ __forceinline__ float coop_pair(const float* x, float fm, float fk, float fq, int p) {
  float v = 0.f, tmin;
  if (pair_range<float>(x[0], x[1], fm, fk, fq, &tmin))
    v = -pair_point<float>(x[0], x[1], fm, fk, fq, tmin, p, x[4]);
  return isfinite(v) ? v : 0.f;
}
__device__ __forceinline__ float coop_photo(const float* x, float fm, float fk, float fq, int p) {
  float v = 0.f, lmin, dx;
  if (photo_range<float>(x[0], x[1], fm, fk, fq, &lmin, &dx))
    v = photo_point<float>(x[0], x[1], fm, fk, fq, lmin, dx, p, x[4]);
  return isfinite(v) ? v : 0.f;
}
__device__ __forceinline__ float coop_bi(const float* x, float fm, float fk, float fq, int t) {
  const float v = t == 0 ? dcs_brems<float>(x[0], x[1], fm, fk, fq, x[4])
                         : dcs_ionisation<float>(x[0], x[2], fm, fk, fq, x[4]);
  return isfinite(v) ? v : 0.f;
}
// Component p of an element from its items `it` (bremsstrahlung, pair,
// photonuclear, ionisation), times the mass fraction and the ancestor energy.
__device__ __forceinline__ float coop_comp(const float* it, int p, float fraction, float fk) {
  float v;
  if (p == 0) {
    v = it[0];
  } else if (p == 1) {
    v = 0.f;
    for (int j = 0; j < 12; ++j) v += it[1 + j];
    v = fmaxf(v, 0.f);
  } else if (p == 2) {
    v = 0.f;
    for (int j = 0; j < 9; ++j) v += it[13 + j];
    v = fmaxf(v, 0.f);
  } else {
    v = it[22];
  }
  v *= fraction * fk;
  return v;
}
// Total of one event's nc components: lane c's running sum of components
// c, c + 32, ..., then a fixed tree over the lanes (lane 0 holds it).
__device__ __forceinline__ float coop_total(const float* comp, int nc, int lane) {
  float mine = 0.f;
  for (int c = lane; c < nc; c += 32) mine += comp[c];
  for (int d = 16; d > 0; d >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, d);
  return mine;
}

// Warp-cooperative FP32 form of del_total for k events of one medium at once
// (their ancestor energies anc[] and transfers q[] in the buffer).  The terms
// of all k events are spread over the lanes one kind at a time (pair
// asymmetry points, photonuclear points, then bremsstrahlung and
// ionisation), so that a pass evaluates one DCS model on up to 32 terms
// instead of four models on one event's 23.  Per event the components are
// summed in a fixed order (kept for the pick) and the total is reduced in a
// fixed tree, so an event's total does not depend on the events served with
// it.  All 32 lanes call it with the same arguments.
static __device__ __noinline__ void coop_batch(const float* elf, int nel, float fm, int k,
                                               float* buf) {
  const int lane = threadIdx.x & 31;
  const int ni = kItemsPerElement * nel, nc = 4 * nel;
  float* item = buf;
  float* comp = item + k * ni;
  float* tot = comp + k * nc;
  const float* anc = buf + coop_head(nel, k);
  const float* q = anc + k;
  for (int f = lane; f < k * nel * 12; f += 32) {
    const int i = f / (nel * 12), r = f - i * nel * 12, e = r / 12, p = r - e * 12;
    item[i * ni + e * kItemsPerElement + 1 + p] = coop_pair(elf + kElfStride * e, fm, anc[i], q[i], p);
  }
  for (int f = lane; f < k * nel * 9; f += 32) {
    const int i = f / (nel * 9), r = f - i * nel * 9, e = r / 9, p = r - e * 9;
    item[i * ni + e * kItemsPerElement + 13 + p] = coop_photo(elf + kElfStride * e, fm, anc[i], q[i], p);
  }
  for (int f = lane; f < k * nel * 2; f += 32) {
    const int i = f / (nel * 2), r = f - i * nel * 2, e = r >> 1, t = r & 1;
    item[i * ni + e * kItemsPerElement + (t ? 22 : 0)] = coop_bi(elf + kElfStride * e, fm, anc[i], q[i], t);
  }
  __syncwarp();
  for (int f = lane; f < k * nc; f += 32) {
    const int i = f / nc, c = f - i * nc, e = c >> 2, p = c & 3;
    comp[i * nc + c] = coop_comp(item + i * ni + e * kItemsPerElement, p, elf[kElfStride * e + 3], anc[i]);
  }
  __syncwarp();
  for (int i = 0; i < k; ++i) {
    const float t = coop_total(comp + i * nc, nc, lane);
    if (lane == 0) tot[i] = t;
  }
  __syncwarp();
}

template <class R>
struct DelOutT {
  R energy, weight;
  int process, element;  // process 0: null CEL event
};
using DelOut = DelOutT<double>;

// reverse_del_event (src/MixedTransport.jl:111-142) up to the DCS sum.  Returns
// true when the event needs that sum; *anc and *denom (pdf r sigma (1 - p_cel))
// then describe it.  Otherwise *out is the result.
template <class R>
static __device__ __noinline__ bool del_begin(const Med<R>& m, const Consts& C, double k, Stream& g,
                                              int* status, DelOut* out, double* anc_out,
                                              double* denom) {
  *out = DelOut{k, 1.0, 0, -1};
  double sigma = double(klookup(m, K_E, K_SIG, R(k), status));
  if (!(sigma > 0.0)) {
    *status |= ST_ZERO_RATE;
    return false;
  }
  double onset = double(m.onset), cut = C.cutoff;
  double pcel = k >= onset ? 0.0 : -log(cut) / (-log(cut) + log(onset / (onset - k)));
  if (pcel > 0.0 && uni_d(g) < pcel) {
    out->weight = 1.0 / pcel;
    return false;
  }
  const double me = kElectronMass, M = C.mass;
  double xmax = k < 0.5 * (M - me) * (M - me) / me
                    ? fmin(1.0, 2.0 * me * (k + 2.0 * M) / ((M + me) * (M + me)))
                    : 1.0;
  double xmin = k >= onset * (1.0 - cut) ? cut : 1.0 - k / onset;
  if (!(xmax > xmin)) return false;
  double invnorm = 1.0 / xmin - 1.0 / xmax;
  double nu = 1.0 / (1.0 / xmin - uni_d(g) * invnorm);
  double rr = 1.0 - nu, anc = k / rr, pdf = 1.0 / (invnorm * nu * nu);
  *anc_out = anc;
  *denom = pdf * rr * sigma * (1.0 - pcel);
  return true;
}
// The same in FP32 for the mixed-precision transport: the same draws and
// decisions, with -log(cutoff) taken from the launch constants,
// log(onset / (onset - k)) as log1p(k / (onset - k)), 1 - nu formed without
// cancellation (for xmax = 1, D - 1 = (1/xmin - 1)(1 - u) with D = 1/nu) and
// the energy transfer as anc nu.  *q receives the transfer.
static __device__ __noinline__ bool del_begin32(const Med<float>& m, const Consts& C, float k, Stream& g,
                                                int* status, DelOutT<float>* out, float* anc_out,
                                                float* q_out, float* denom) {
  *out = DelOutT<float>{k, 1.f, 0, -1};
  const float sigma = klookup(m, K_E, K_SIG, k, status);
  if (!(sigma > 0.f)) {
    *status |= ST_ZERO_RATE;
    return false;
  }
  const float onset = m.onset, cut = C.cutoff_f, lc = C.lcut_f;
  const float pcel = k >= onset ? 0.f : lc / (lc + log1pf(k / (onset - k)));
  if (pcel > 0.f && uni<float>(g) < pcel) {
    out->weight = 1.f / pcel;
    return false;
  }
  const float me = float(kElectronMass), M = C.mass_f;
  const float xmax = k < 0.5f * (M - me) * (M - me) / me
                         ? fminf(1.f, 2.f * me * (k + 2.f * M) / ((M + me) * (M + me)))
                         : 1.f;
  const float xmin = k >= onset * (1.f - cut) ? cut : 1.f - k / onset;
  if (!(xmax > xmin)) return false;
  const float ixmin = 1.f / xmin, invnorm = ixmin - 1.f / xmax;
  const float u = uni<float>(g);
  const float D = ixmin - u * invnorm, nu = 1.f / D;
  const float rr = xmax >= 1.f ? invnorm * (1.f - u) / D : 1.f - nu;
  const float anc = k / rr;
  *anc_out = anc;
  *q_out = anc * nu;
  *denom = rr * sigma * (1.f - pcel) / (invnorm * nu * nu);
  return true;
}
// The rest of reverse_del_event once the DCS sum (and, with details, the
// picked component) is known.
template <class R>
__device__ __forceinline__ DelOutT<R> del_end(R anc, R denom, R total, int pick) {
  DelOutT<R> r{anc, total / denom, 0, -1};
  if (pick >= 0) {
    r.process = pick % 4 + 1;
    r.element = pick / 4;
  }
  return r;
}
// reverse_del_event in one thread, FP64 (src/MixedTransport.jl:111-142).
template <class R>
static __device__ __noinline__ DelOut reverse_del(const Med<R>& m, const Consts& C, double k, Stream& g,
                                           bool details, int* status) {
  DelOut r;
  double anc, denom;
  if (!del_begin(m, C, k, g, status, &r, &anc, &denom)) return r;
  double total = del_total(m.el, m.nel, C.mass, anc, anc - k);
  int pick = -1;
  if (details && total > 0.0) pick = del_pick(m.el, m.nel, C.mass, anc, anc - k, uni_d(g) * total);
  return del_end(anc, denom, total, pick);
}

// Altitude of a history and of the layer boundaries.  FP64 transport: a
// double.  FP32 transport: an unevaluated pair hi + lo of floats updated by
// compensated sums (about 48 bits), so that the step loop needs no FP64
// instruction (FP64 issues at 1/64 of the FP32 rate on this GPU).  Only the
// altitude enters the transport; the horizontal position is not tracked.
template <class R> struct AltT;
template <> struct AltT<double> { using type = double; };
template <> struct AltT<float> { using type = F2; };
template <class R> using Alt = typename AltT<R>::type;

__device__ __forceinline__ double alt_value(double z) { return z; }
__device__ __forceinline__ double alt_value(F2 z) { return double(z.h) + double(z.l); }
template <class R> __device__ __forceinline__ Alt<R> alt_make(double v);
template <> __device__ __forceinline__ double alt_make<double>(double v) { return v; }
template <> __device__ __forceinline__ F2 alt_make<float>(double v) {
  float h = float(v);
  return F2{h, float(v - double(h))};
}
// z += dz
__device__ __forceinline__ void alt_add(double& z, double dz) { z += dz; }

// Mutable part of a history.
template <class R>
struct State {
  Alt<R> z;
  R ux, uy, uz, E, w;
  int status;
};

// A step suspended on a hard-event DCS sum (cooperative evaluation): what it
// needs to resume.  Mixed step: a = remaining, b = travelled, c = density,
// d = round-off floor, r0 = energy, r1 = weight, r2 = ceiling, event.
// Straggled step: a = requested length, r0 = initial energy, r1 = event
// energy, r2 = event grammage, r3 = density, flag = scattering.
template <class R>
struct Cont {
  R a, b, c, d, dist;  // dist: requested length of a mixed step
  R moved;             // path length of a completed straggled step (when asked)
  R r0, r1, r2, r3;
  int event, kind, medium, flag;
  R anc, q, denom;  // the pending event: ancestor, energy transfer, weight denominator
  int details;
  R total;          // answer: DCS sum and picked component
  int pick;
};
enum : int { CONT_NONE = 0, CONT_MIXED = 1, CONT_STRAG = 2 };

// Path length of a completed mixed step: FP64, travelled grammage / density as
// the reference (src/MixedTransport.jl:198); FP32, the requested length when
// the segment was consumed.
template <class R>
__device__ __forceinline__ R mixed_moved(const Cont<R>& x) {
  return (sizeof(R) == 4 && x.a <= x.d) ? x.dist : x.b / x.c;
}

// transport_mixed_step (src/MixedTransport.jl:144-200), resumable.  The
// round-off floor of the grammage bookkeeping is the reference's FP64
// eps(max(1, grammage)) in both precisions: an FP32 ulp would exceed the
// grammage of the 1e-7 m boundary-crossing steps.
template <class R>
__device__ void mixed_end(State<R>& s, const Cont<R>& x, R Emax, R energy_limit, bool exhausted) {
  if (exhausted) s.status |= ST_EVENT_CAP;
  if (x.r1 > R(0) && x.r0 >= Emax && x.a > x.d && (energy_limit < R(0) || x.r0 < energy_limit))
    s.status |= ST_DOMAIN_HI;
  s.E = x.r0;
  s.w = x.r1;
  alt_add(s.z, -(mixed_moved(x) * s.uz));
}
// Applies a hard event; true when the history's weight vanished.
template <class R>
__device__ __forceinline__ bool mixed_event(State<R>& s, Cont<R>& x, const DelOutT<R>& d) {
  x.r0 = d.energy;
  x.r1 = x.r1 * d.weight;
  if (!(isfinite(x.r1) && x.r1 >= R(0))) s.status |= ST_BAD_WEIGHT;
  return x.r1 == R(0);
}
// Runs the event loop from x.event; returns true when it suspended on a DCS sum.
// The per-step helpers (mixed_run, fluctuate, straggled_end) come in two
// forms: *_in, inlined into the caller, and an out-of-line function.  The
// two-layer transport's straggled steps call them out of line (that step body
// is large and bound by instruction fetch); its mixed phase (mixed steps only)
// and the fixed-path transport, which never scatters, inline them.
template <class R, bool COOP>
__device__ __forceinline__ bool mixed_run_in(const Med<R>& m, const Consts& C, State<R>& s, Cont<R>& x,
                                             Stream& g, R energy_limit) {
  const int nk = m.nk;
  const R* kE = m.kcol(K_E);
  const R Emax = kE[nk - 1];
  const R mass = C.mass_r<R>(), ctau = C.ctau_r<R>(), rdens = x.c;
  for (; x.event < C.event_cap; ++x.event) {
    R k = x.r0;
    if (x.a <= x.d || k >= x.r2) {
      mixed_end(s, x, Emax, energy_limit, false);
      return false;
    }
    KLoc<R> Lk = klocate_e(m, k, &s.status);
    R ri = kat(m.kcol(K_R), nk, Lk), hi = kat(m.kcol(K_H), nk, Lk);
    R rtc = fmax(R(0), klookup(m, K_E, K_R, x.r2, &s.status) - ri);
    R eg = fmin(x.a, rtc);
    R endpoint = eg == rtc ? x.r2 : fmax(k, klookup(m, K_R, K_E, ri + eg, &s.status));
    R eventh = hi + expo<R>(g);
    bool occurs = eventh < klookup(m, K_E, K_H, endpoint, &s.status);
    R pre = occurs ? fmax(k, klookup(m, K_H, K_E, eventh, &s.status)) : endpoint;
    KLoc<R> Lp = klocate_e(m, pre, &s.status);
    R dx = occurs ? fmax(R(0), kat(m.kcol(K_R), nk, Lp) - ri) : eg;
    R dt;
    if (dx <= R(8) * ulp_up(fabs(ri)) || pre - k <= R(8) * ulp_up(fabs(k)))
      dt = dx / x.c * mass / R(2) *
           (R(1) / sqrt(k * (k + R(2) * mass)) + R(1) / sqrt(pre * (pre + R(2) * mass)));
    else
      dt = (kat(m.kcol(K_T), nk, Lp) - kat(m.kcol(K_T), nk, Lk)) / rdens;
    x.r1 *= kat(m.kcol(K_S), nk, Lp) / kat(m.kcol(K_S), nk, Lk) * exp(-dt / ctau);
    x.b += dx;
    x.a = fmax(R(0), x.a - dx);
    x.r0 = pre;
    if (!occurs) {
      mixed_end(s, x, Emax, energy_limit, false);
      return false;
    }
    DelOutT<R> d;
    if constexpr (COOP) {  // FP32
      if (del_begin32(m, C, pre, g, &s.status, &d, &x.anc, &x.q, &x.denom)) {
        x.details = 0;
        return true;
      }
    } else {  // FP64
      d = reverse_del(m, C, double(pre), g, false, &s.status);
    }
    if (mixed_event(s, x, d)) {
      mixed_end(s, x, Emax, energy_limit, false);
      return false;
    }
  }
  mixed_end(s, x, Emax, energy_limit, true);
  return false;
}
template <class R, bool COOP>
static __device__ __noinline__ bool mixed_run(const Med<R>& m, const Consts& C, State<R>& s, Cont<R>& x,
                                              Stream& g, R energy_limit) {
  return mixed_run_in<R, COOP>(m, C, s, x, g, energy_limit);
}
// Starts a mixed step of `distance` m at `density`; true when it suspended.
template <class R, bool COOP, bool INL = false>
__device__ bool mixed_step(const Med<R>& m, const Consts& C, State<R>& s, R density, R distance,
                           Stream& g, R energy_limit, Cont<R>& x) {
  const R Emax = m.kcol(K_E)[m.nk - 1];
  if (s.E > Emax) {
    s.status |= ST_DOMAIN_HI;
    return false;
  }
  x.a = distance * density;
  x.b = R(0);
  x.c = density;
  x.dist = distance;
  const R dXreq = fmax(R(1), distance * density);
  if (sizeof(R) == 8) x.d = ulp_up(dXreq);
  else x.d = dXreq * R(2.220446049250313e-16);
  x.r0 = s.E;
  x.r1 = s.w;
  x.r2 = energy_limit > R(0) ? fmin(energy_limit, Emax) : Emax;
  x.event = 0;
  if constexpr (INL) return mixed_run_in<R, COOP>(m, C, s, x, g, energy_limit);
  else return mixed_run<R, COOP>(m, C, s, x, g, energy_limit);
}

// ------------------------------------------------------------ straggling
template <class R>
__device__ __forceinline__ R box_muller(Stream& g) {
  R r = sqrt(R(-2) * log(uni<R>(g)));
  R phi = R(2) * R(kPi) * uni<R>(g);
  return r * sin(phi);
}
template <class R>
__device__ __forceinline__ R truncated_randn(Stream& g) {
  R u = box_muller<R>(g);
  for (int it = 0; it < 1000 && fabs(u) > R(3); ++it) u = box_muller<R>(g);
  return u * R(0.9848416472);
}

// fluctuate_energy_loss, backward (src/Straggling.jl:103-173, :1046-1105).
template <class R>
__device__ __forceinline__ R fluctuate_in(const Med<R>& m, R ki, const Loc<R>& Li, R dX, R Xtot,
                                        Stream& g, R* ratio_out) {
  R k1 = inv_range(m, MC_MR, Xtot + dX);
  R dk0 = fabs(ki - k1), ratio = R(1);
  if (k1 > R(0) && dk0 > R(0)) {
    Loc<R> L1 = locate(m, k1);
    R O0 = at(m, Li, MC_STRAG), O1 = at(m, L1, MC_STRAG);
    R dk12 = R(0.5) * dX * (O0 + O1);
    if (dX / Xtot > R(0.05)) {
      R de1 = at(m, L1, MC_MS), de0 = at(m, Li, MC_MS);
      dk12 *= R(1) - dX / dk0 * (de1 - de0);
    }
    R dk1 = sqrt(fmax(dk12, R(0)));
    if (dk0 >= R(3) * dk1 && dk1 > R(0)) {
      k1 += truncated_randn<R>(g) * dk1;
    } else if (dk0 >= R(1.7320508) * dk1 && dk1 > R(0)) {
      k1 += R(1.7320508) * (R(1) - R(2) * uni<R>(g)) * dk1;
    } else if (dk1 > R(0)) {
      R dk32 = R(3) * dk12, dk02 = dk0 * dk0;
      R a = R(1) - (dk32 - dk02) / (dk32 + R(3) * dk02);
      if (uni<R>(g) <= a) {
        R b = R(0.5) * (dk32 + R(3) * dk02) / dk0;
        k1 = ki + b * uni<R>(g);
        if (k1 < R(0)) k1 = R(0);
      } else {
        k1 = ki;
      }
    }
    ratio = fabs(ki - k1) / dk0;
  }
  if (ratio == R(0)) ratio = R(1);
  *ratio_out = ratio;
  return fmax(k1, R(0));
}
template <class R>
static __device__ __noinline__ R fluctuate(const Med<R>& m, R ki, const Loc<R>& Li, R dX, R Xtot, Stream& g,
                                           R* ratio_out) {
  return fluctuate_in<R>(m, ki, Li, dX, Xtot, g, ratio_out);
}

// sample_ehs_event, backward (src/Straggling.jl:373-434, :1284-1334).
template <class R>
static __device__ __noinline__ bool ehs_event(const Med<R>& m, R ki, R kf, R dX, R Xtot, R ratio, Stream& g, R mass,
                          R eratio, R* X_ehs, R* k_ehs) {
  R kmin = fmin(ki, kf), kmax = fmax(ki, kf);
  if (kmin < R(0.001)) {
    R t = kmin;
    kmin = kmax;
    kmax = t;
  }
  R lb = ehs_path(m, kmin, mass, eratio);
  if (lb <= R(0) || lb >= R(kEhsPathMax)) return false;
  R zeta = uni<R>(g);
  if (zeta <= R(0) || zeta >= R(1)) return false;
  R X = -log(zeta) * lb;
  if (X >= dX) return false;
  R kh = inv_range(m, MC_MR, Xtot + X);
  R k = ki + ratio * fabs(ki - kh);
  if (k <= R(0)) return false;
  R lbk = ehs_path(m, k, mass, eratio);
  if (lbk <= R(0) || lbk >= R(kEhsPathMax)) return false;
  R r = lbk / lb;
  if (r <= R(0) || uni<R>(g) > R(1) / r) return false;
  *X_ehs = X;
  *k_ehs = k;
  return true;
}

// sample_scattering_angle (src/Straggling.jl:446-517, :1344-1405), FP64.
template <class R>
static __device__ __noinline__ double scattering_angle(const Med<R>& m, double mass, double K,
                                                Stream& g) {
  Loc<R> L = locate(m, R(K));
  double p2 = K * (K + 2.0 * mass);
  double mu0 = fmax(double(at(m, L, MC_MU0)), 1e-12);
  double zoa = double(m.ZoA);
  double At = zoa > 0.0 ? 1.0 / zoa : 22.0, Mt = At * kNeutronMass;
  double s = mass * mass + Mt * Mt + 2.0 * (K + mass) * Mt;
  double K0 = (s - (mass + Mt) * (mass + Mt)) / (2.0 * sqrt(s));
  double Ecm = K0 + mass, pcm = sqrt(fmax(K0 * (K0 + 2.0 * mass), 0.0));
  double El = K + mass, pl = sqrt(fmax(p2, 0.0));
  double gCM = (pl > 0.0 && pcm > 0.0) ? (El * Ecm + pl * pcm) / (mass * sqrt(s)) : 1.0;
  double tau = (pl > 0.0 && pcm > 0.0) ? (El * pcm - Ecm * pl) / (pl * pcm) : 0.0;
  double A = mu0 / 4.0, fs = double(at(m, L, MC_FSPIN));
  double Apm = A + mu0, Ap1 = A + 1.0, omm = 1.0 - mu0, mu1 = mu0;
  for (int it = 0; it < 100; ++it) {
    double zeta = uni_d(g);
    double tmp = Ap1 - zeta * omm;
    if (tmp <= 0.0) continue;
    double tr = fmin(fmax(Apm * Ap1 / tmp - A, mu0), 1.0);
    if (uni_d(g) <= 1.0 - fs * tr) {
      mu1 = tr;
      break;
    }
  }
  double mu;
  if (mu1 > 1e-6) {
    double a = gCM * (tau + 1.0 - 2.0 * mu1);
    double ct = a / sqrt(4.0 * mu1 * (1.0 - mu1) + a * a);
    mu = 0.5 * (1.0 - ct);
  } else {
    double d = gCM * (1.0 + tau);
    mu = mu1 / (d * d);
  }
  return fmin(fmax(mu, 0.0), 1.0);
}

// FP32 form of scattering_angle for the mixed-precision transport.  The CM
// kinetic energy uses the exact identity s - (m + M)^2 = 2 K M instead of the
// difference (which cancels in FP32 at low energy).
static __device__ __noinline__ float scattering_angle_f(const Med<float>& m, float mass, float K,
                                                 Stream& g) {
  Loc<float> L = locate(m, K);
  float p2 = K * (K + 2.f * mass);
  float mu0 = fmaxf(at(m, L, MC_MU0), 1e-12f);
  float zoa = m.ZoA;
  float At = zoa > 0.f ? 1.f / zoa : 22.f, Mt = At * float(kNeutronMass);
  float s = mass * mass + Mt * Mt + 2.f * (K + mass) * Mt, rs = sqrtf(s);
  float K0 = K * Mt / rs;
  float Ecm = K0 + mass, pcm = sqrtf(fmaxf(K0 * (K0 + 2.f * mass), 0.f));
  float El = K + mass, pl = sqrtf(fmaxf(p2, 0.f));
  float gCM = (pl > 0.f && pcm > 0.f) ? (El * Ecm + pl * pcm) / (mass * rs) : 1.f;
  float tau = (pl > 0.f && pcm > 0.f) ? (El * pcm - Ecm * pl) / (pl * pcm) : 0.f;
  float A = mu0 * 0.25f, fs = at(m, L, MC_FSPIN);
  float Apm = A + mu0, Ap1 = A + 1.f, omm = 1.f - mu0, mu1 = mu0;
  for (int it = 0; it < 100; ++it) {
    float zeta = uni<float>(g);
    float tmp = Ap1 - zeta * omm;
    if (tmp <= 0.f) continue;
    float tr = fminf(fmaxf(Apm * Ap1 / tmp - A, mu0), 1.f);
    if (uni<float>(g) <= 1.f - fs * tr) {
      mu1 = tr;
      break;
    }
  }
  float mu;
  if (mu1 > 1e-6f) {
    float a = gCM * (tau + 1.f - 2.f * mu1);
    float ct = a / sqrtf(4.f * mu1 * (1.f - mu1) + a * a);
    mu = 0.5f * (1.f - ct);
  } else {
    float d = gCM * (1.f + tau);
    mu = mu1 / (d * d);
  }
  return fminf(fmaxf(mu, 0.f), 1.f);
}

// sample_soft_scattering (src/Straggling.jl:539-590, :1204-1253).  lb0 is
// the transport path at the step's start (the step limit computed it) and
// L1 the location of k1 (the weight update uses it too).
template <class R>
static __device__ __noinline__ R soft_scattering(const Med<R>& m, R lb0, const Loc<R>& L1, R k1,
                                                 R step, R density, Stream& g) {
  if (step <= R(0) || density <= R(0)) return R(0);
  R inv0 = lb0 > R(0) ? density / lb0 : R(0), inv1;
  if (k1 > R(0)) {
    R lb1 = transport_path(m, L1);
    inv1 = lb1 > R(0) ? density / lb1 : R(0);
  } else {
    inv1 = inv0;
  }
  if (inv0 <= R(0) && inv1 <= R(0)) return R(0);
  R ilb1 = R(0.25) * step * (inv0 + inv1);
  if (ilb1 < R(1e-12)) return R(0);
  if (ilb1 > R(1)) ilb1 = R(1);
  for (int it = 0; it < 1000; ++it) {
    R u = uni<R>(g);
    if (!(u > R(0))) continue;
    R mu = -ilb1 * log(u);
    if (mu <= R(1)) return fmax(mu, R(0));
  }
  return ilb1;
}

// rotate_direction (src/Straggling.jl:645-710).
template <class R>
static __device__ __noinline__ void rotate(State<R>& s, R mu, Stream& g) {
  R ct = R(1) - R(2) * mu, st2 = R(4) * mu * (R(1) - mu);
  if (st2 <= R(0)) return;
  R st = sqrt(st2), d0 = s.ux, d1 = s.uy, d2 = s.uz;
  R ax = fabs(d0), ay = fabs(d1), az = fabs(d2);
  R u0x = R(0), u0y = R(0), u0z = R(0);
  if (ax > ay) {
    if (ax > az) {
      R nrm = R(1) / sqrt(d0 * d0 + d2 * d2);
      u0x = -d2 * nrm;
      u0z = d0 * nrm;
    } else {
      R nrm = R(1) / sqrt(d1 * d1 + d2 * d2);
      u0y = d2 * nrm;
      u0z = -d1 * nrm;
    }
  } else {
    if (ay > az) {
      R nrm = R(1) / sqrt(d0 * d0 + d1 * d1);
      u0x = d1 * nrm;
      u0y = -d0 * nrm;
    } else {
      R nrm = R(1) / sqrt(d1 * d1 + d2 * d2);
      u0y = d2 * nrm;
      u0z = -d1 * nrm;
    }
  }
  R u1x = u0y * d2 - u0z * d1, u1y = u0z * d0 - u0x * d2, u1z = u0x * d1 - u0y * d0;
  R cp, sp;
  sincospi(R(1) - R(2) * uni<R>(g), &sp, &cp);
  R nx = ct * d0 + st * (cp * u0x + sp * u1x);
  R ny = ct * d1 + st * (cp * u0y + sp * u1y);
  R nz = ct * d2 + st * (cp * u0z + sp * u1z);
  R nrm = sqrt(nx * nx + ny * ny + nz * nz);
  if (nrm > R(0)) {
    nx /= nrm;
    ny /= nrm;
    nz /= nrm;
  }
  s.ux = nx;
  s.uy = ny;
  s.uz = nz;
}

// DEL polar angles, FP64 (src/Straggling.jl:746-914).
static __device__ __noinline__ double polar_brems(double m, double ki, double kf, double RN, Stream& g) {
  double E = ki + m, nu = ki - kf;
  if (nu <= 0.0 || E <= m) return 0.0;
  double y = nu / E, tmp = 0.5 * m * nu / (E * (E - nu)), mu0 = tmp * tmp;
  double c1 = (2.0 * (1.0 - y) + y * y) * mu0, c2 = 4.0 * (1.0 - y) * mu0 * mu0;
  double t2 = m * RN / kHbarC, muni = t2 * t2 / 6.0;
  if (sqrt(mu0) - mu0 < 0.0) return 0.0;
  double q0 = muni, r0 = mu0, qr0 = q0 * r0, den0 = r0 + qr0;
  if (den0 <= 0.0 || (1.0 + qr0) <= 0.0) return 0.0;
  double x0 = (1.0 + 2.0 * qr0) * log((1.0 + qr0) / den0) - (1.0 - r0) * (1.0 + 2.0 * q0) / (1.0 + q0);
  if (x0 <= 0.0) return 0.0;
  for (int it = 0; it < 100; ++it) {
    double r0r = uni_d(g), r1 = uni_d(g);
    double mu = r0r * mu0 / (mu0 + 1.0 - r0r);
    double mus = mu0 + mu, mu2 = mus * mus, d1 = 1.0 / mu2, d2 = d1 * d1;
    double score = r1 * c1 * d1, pdf = c1 * d1 - mu * c2 * d2;
    if (score > pdf) continue;
    double l2 = mu2 / (mu0 * mu0), q = muni * l2, r = mu0 * l2, qr = q * r;
    if (qr > 1e5) continue;
    double den = r + qr;
    if (den <= 0.0 || (1.0 + qr) <= 0.0) continue;
    double x = (1.0 + 2.0 * qr) * log((1.0 + qr) / den) - (1.0 - r) * (1.0 + 2.0 * q) / (1.0 + q);
    pdf *= x / x0;
    if (score <= pdf) return mu;
  }
  return 0.0;
}
// The same in FP32, with every term scaled by the smallest angle mu0: in
// units of mu0 the density and the score stay of order one (their FP64 form
// reaches mu0^-4, beyond the FP32 range for small mu0).  t = mu / mu0 and
// s = 1 + t; the draws are the same.
static __device__ __noinline__ float polar_brems32(float m, float ki, float kf, float RN, Stream& g) {
  const float E = ki + m, nu = ki - kf;
  if (nu <= 0.f || E <= m) return 0.f;
  const float y = nu / E, tmp = 0.5f * m * nu / (E * (E - nu)), mu0 = tmp * tmp;
  const float C1 = 2.f * (1.f - y) + y * y, C2 = 4.f * (1.f - y);
  const float t2 = m * RN / float(kHbarC), muni = t2 * t2 / 6.f;
  if (sqrtf(mu0) - mu0 < 0.f) return 0.f;
  const float qr0 = muni * mu0, den0 = mu0 + qr0;
  if (den0 <= 0.f || (1.f + qr0) <= 0.f) return 0.f;
  const float x0 = (1.f + 2.f * qr0) * logf((1.f + qr0) / den0) -
                   (1.f - mu0) * (1.f + 2.f * muni) / (1.f + muni);
  if (x0 <= 0.f) return 0.f;
  for (int it = 0; it < 100; ++it) {
    const float r0r = uni<float>(g), r1 = uni<float>(g);
    const float t = r0r / (mu0 + 1.f - r0r), sc = 1.f + t, s2 = sc * sc;
    const float score = r1 * C1 / s2;
    float pdf = C1 / s2 - t * C2 / (s2 * s2);
    if (score > pdf) continue;
    const float q = muni * s2, r = mu0 * s2, qr = q * r;
    if (qr > 1e5f) continue;
    const float den = r + qr;
    if (den <= 0.f || (1.f + qr) <= 0.f) continue;
    const float x = (1.f + 2.f * qr) * logf((1.f + qr) / den) - (1.f - r) * (1.f + 2.f * q) / (1.f + q);
    pdf *= x / x0;
    if (score <= pdf) return t * mu0;
  }
  return 0.f;
}
static __device__ __noinline__ double polar_photo(double ml, double ki, double kf, Stream& g) {
  double M = 0.5 * (kProtonMass + kNeutronMass), q = ki - kf, E = ki + ml, ml2 = ml * ml;
  double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
  double Q2max = 2.0 * M * (q - kPionMass) - kPionMass * kPionMass;
  if (Q2max < Q2min || Q2min < 0.0) return 0.0;
  double rQ2 = log(Q2max) - log(Q2min);
  double Q2 = Q2min * exp(rQ2 * uni_d(g));
  double p = sqrt(ki * (ki + 2.0 * ml)), E1 = E - q, er = ml / E1;
  double p1 = E1 * sqrt(fmax((1.0 + er) * (1.0 - er), 0.0)), p2 = p * p1;
  if (p2 <= 0.0) return 0.0;
  double tv = p2 + ml2 - E * E1;
  if (fabs(tv) <= 3.0 * kEps64 * p2) tv = 0.0;
  double mu = 0.5 * tv / p2 + 0.25 / p2 * Q2;
  return fmin(fmax(mu, 0.0), 1.0);
}
__device__ __forceinline__ double polar_ioni(double m, double ki, double kf) {
  double nu = ki - kf, p2 = ki * (ki + 2.0 * m), E = ki + m;
  double den = sqrt(p2 * (p2 + nu * nu - 2.0 * nu * E));
  if (den <= 0.0) return 0.0;
  double c = (p2 - nu * (E + kElectronMass)) / den;
  return 0.5 * (1.0 - c);
}

// transport_backward_step_full, mode :straggled (src/Geometry.jl:148-357):
// straggled_end completes a step from its energy-loss and event decisions.
template <class R>
__device__ __forceinline__ R straggled_end_in(const Med<R>& m, const Consts& C, State<R>& s,
                                              const Loc<R>& Li, R lb0, R ki, R kf, R ckf, R dX,
                                              R dw,
                                              int proc, int elem, bool del, bool ehs, R k_ehs,
                                              R density, R step, bool shortened, bool scattering,
                                              Stream& g) {
  const R mass = C.mass_r<R>();
  R astep = dX / density;
  R oz = s.uz;  // the position moves along the incoming direction
  const Loc<R> Lc = locate(m, ckf);  // soft scattering and the weight update
  if (scattering) {
    if (del && proc > 0) {
      R mu;
      if (proc == 1 || proc == 2) {
        if constexpr (sizeof(R) == 8)
          mu = polar_brems(C.mass, kf, ckf, m.el[kElStride * elem + 4], g);
        else
          mu = polar_brems32(C.mass_f, kf, ckf, m.elf[kElfStride * elem + 5], g);
      } else {
        mu = R(proc == 3 ? polar_photo(C.mass, double(kf), double(ckf), g)
                         : polar_ioni(C.mass, double(kf), double(ckf)));
      }
      if (mu > R(0)) rotate(s, mu, g);
    }
    if (ehs) {
      R mu;
      if constexpr (sizeof(R) == 4) mu = scattering_angle_f(m, mass, k_ehs, g);
      else mu = R(scattering_angle(m, C.mass, double(k_ehs), g));
      if (mu > R(0)) rotate(s, mu, g);
    }
    R mu = soft_scattering(m, lb0, Lc, ckf, astep, density, g);
    if (mu > R(0)) rotate(s, mu, g);
  }
  R pt = astep * mass / R(2) *
         (R(1) / sqrt(ki * (ki + R(2) * mass)) + R(1) / sqrt(ckf * (ckf + R(2) * mass)));
  // FP64: the reference's dX/density; FP32: the requested FP64 step unless
  // an event or the energy limit shortened it
  R da = astep;
  if (sizeof(R) == 4) da = shortened ? dX / density : step;
  alt_add(s.z, -(da * oz));
  R wf = at(m, Lc, MC_MS) / at(m, Li, MC_MS);
  if (sizeof(R) == 4) s.w = s.w * wf * exp(-pt / C.ctau_r<R>()) * dw;
  else s.w = R(double(s.w * wf * exp(-pt / C.ctau_r<R>())) * dw);
  s.E = kf;
  return da;
}
template <class R>
static __device__ __noinline__ R straggled_end(const Med<R>& m, const Consts& C, State<R>& s, const Loc<R>& Li,
                                               R lb0, R ki, R kf, R ckf, R dX, R dw, int proc,
                                               int elem, bool del, bool ehs, R k_ehs, R density,
                                               R step, bool shortened, bool scattering, Stream& g) {
  return straggled_end_in<R>(m, C, s, Li, lb0, ki, kf, ckf, dX, dw, proc, elem, del, ehs, k_ehs,
                             density, step, shortened, scattering, g);
}

// The step up to its hard-event decision; true when it suspended on the
// event's DCS sum (cooperative evaluation), with x holding what straggled_end
// needs.
// With MOVED, x.moved receives the path length of a completed step.
template <class R, bool COOP, bool MOVED = false, bool INL = false>
__device__ bool straggled_step(const Med<R>& m, const Consts& C, State<R>& s, const Loc<R>& Li,
                               R lb0, R density, R step, Stream& g, bool scattering,
                               R energy_limit, Cont<R>& x) {
  const R mass = C.mass_r<R>(), eratio = C.eratio_r<R>();
  R ki = s.E, dX = step * density;
  bool shortened = false;  // the step ended before its requested length
  R Xi = at(m, Li, MC_MR);
  R kf = ki, ratio = R(1);
  if (ki > R(0.001)) {
    if constexpr (INL) kf = fluctuate_in(m, ki, Li, dX, Xi, g, &ratio);
    else kf = fluctuate(m, ki, Li, dX, Xi, g, &ratio);
    kf = fmax(kf, ki);
  } else {
    kf = inv_range(m, MC_MR, Xi + dX);
  }
  if (energy_limit > R(0) && kf >= energy_limit) {
    R dk = fabs(ki - kf);
    if (dk > R(0)) {
      dX = dX * (fabs(energy_limit - ki) / dk);
      kf = energy_limit;
      shortened = true;
    }
  }
  bool del = false, ehs = false;
  R X_del = R(CUDART_INF), k_del = R(0), X_ehs = R(CUDART_INF), k_ehs = R(0);
  R rate = fmax(klookup(m, K_E, K_SIG, ki, &s.status), klookup(m, K_E, K_SIG, kf, &s.status));
  if (rate > R(0)) {
    R cand = expo<R>(g) / rate;
    if (cand < dX) {
      R kh = inv_range(m, MC_MR, Xi + cand);
      R pre = ki + ratio * fabs(kh - ki);
      if (pre > R(0) && uni<R>(g) <= klookup(m, K_E, K_SIG, pre, &s.status) / rate) {
        del = true;
        X_del = cand;
        k_del = pre;
      }
    }
  }
  if (scattering) {
    R X, k;
    if (ehs_event(m, ki, kf, dX, Xi, ratio, g, mass, eratio, &X, &k) && k > R(0)) {
      ehs = true;
      X_ehs = X;
      k_ehs = k;
    }
  }
  if (del && ehs) {
    if (X_del <= X_ehs) ehs = false;
    else del = false;
  }
  R dw = R(1);
  R ckf = kf;
  int proc = 0, elem = -1;
  if (del) {
    DelOutT<R> d;
    if constexpr (COOP) {  // FP32
      if (del_begin32(m, C, k_del, g, &s.status, &d, &x.anc, &x.q, &x.denom)) {
        x.details = 1;
        x.a = step;
        x.r0 = ki;
        x.r1 = k_del;
        x.r2 = X_del;
        x.r3 = density;
        x.flag = scattering;
        return true;
      }
    } else {  // FP64
      d = reverse_del(m, C, double(k_del), g, true, &s.status);
    }
    ckf = k_del;
    kf = d.energy;
    dw = d.weight;
    proc = d.process;
    elem = d.element;
    dX = X_del;
    shortened = true;
  }
  if (ehs) {
    kf = k_ehs;
    ckf = k_ehs;
    dX = X_ehs;
    shortened = true;
  }
  R moved;
  if constexpr (INL)
    moved = straggled_end_in(m, C, s, Li, lb0, ki, kf, ckf, dX, dw, proc, elem, del, ehs, k_ehs, density,
                             step, shortened, scattering, g);
  else
    moved = straggled_end(m, C, s, Li, lb0, ki, kf, ckf, dX, dw, proc, elem, del, ehs, k_ehs, density,
                          step, shortened, scattering, g);
  if (MOVED) x.moved = moved;
  return false;
}

// Deterministic CSDA step on a medium (src/Geometry.jl:424-457).
template <class R>
__device__ __forceinline__ void csda_step(const Med<R>& m, const Consts& C, State<R>& s,
                                          const Loc<R>& Li, R density, R step) {
  const R mass = C.mass_r<R>();
  R ki = s.E, dX = step * density;
  R kf = inv_range(m, MC_CR, at(m, Li, MC_CR) + dX);
  R gm = (R(1) + ki / mass + R(1) + kf / mass) / R(2);
  R b = sqrt(fmax(R(1) - R(1) / (gm * gm), R(1e-12)));
  R dt = step / (b * gm);
  alt_add(s.z, -(step * s.uz));
  s.w = s.w * (at(m, locate(m, kf), MC_CS) / at(m, Li, MC_CS)) * exp(-dt / C.ctau_r<R>());
  s.E = kf;
}

// One history in flight: the state plus its position in the dual-mode loop
// of src/Geometry.jl:534-672, flattened so that a thread can refill itself
// with a new history as soon as the current one ends.
template <class R>
struct Hist {
  State<R> s;
  R limit;  // energy limit of the current mode (exactly representable in R)
  Alt<R> thick, H;
  R rho;
  int steps, inner, outer;
  bool need_mode, strag, mixed, scat;
  Cont<R> x;     // suspended step, if x.kind != CONT_NONE
};
// A history of the two-layer geometry with the shallow porous layer of
// TwoLayerGeometry (src/Geometry.jl:47-72): the porous material at density
// prho for z in [pz, thick); pz = thick when the layer is absent.
template <class R>
struct HistP : Hist<R> {
  Alt<R> pz;
  R prho;
};

enum : int { ADV_STEP = 0, ADV_DONE = 1, ADV_WAIT = 2, ADV_HANDOFF = 3 };

// The transport runs in two persistent phases: PHASE 0 below the mode switch
// (straggled or CSDA steps), PHASE 1 above it (mixed or CSDA steps).  The
// energy never decreases in backward transport, so a history crosses the
// switch once; phase 0 hands it over (ADV_HANDOFF) through a queue in HBM.
// Each phase's loop then holds one step type, not all of them.

// Bookkeeping after a completed step.
template <class R>
__device__ __forceinline__ int step_done(Hist<R>& h, const Consts& C) {
  ++h.inner;
  if (++h.steps > C.step_cap) h.s.status |= ST_STEP_CAP;
  return (h.s.status & ST_FATAL) != 0 ? ADV_DONE : ADV_STEP;
}

// Advances a history by one transport step: ADV_STEP, ADV_DONE when it has
// ended, ADV_WAIT when the step suspended on a hard-event DCS sum.
// Geometry of the current step (src/Geometry.jl:553-650): whether the
// history has left the column, the medium, the distance to the boundary
// ahead and the local density.  FP64: the reference's operations on doubles;
// FP32: the altitude pairs and FP32 arithmetic.
__device__ __forceinline__ bool outside(double z, double H) {
  return z < 0.0 || z >= H - kEps64;
}
__device__ __forceinline__ bool outside(F2 z, F2 H) {
  return z.h + z.l < 0.f || alt_sub(z, H) >= 0.f;
}
__device__ __forceinline__ bool in_air_at(double z, double thick) { return z >= thick; }
__device__ __forceinline__ bool in_air_at(F2 z, F2 thick) { return alt_sub(z, thick) >= 0.f; }
__device__ __forceinline__ void boundary(double z, double thick, double H, bool in_air, double uz,
                                         double rho, double* tob, double* dens) {
  const double eps = kEps64;
  if (!in_air) {
    *dens = rho;
    *tob = uz > eps ? (thick - z) / uz : uz < -eps ? (0.0 - z) / uz : 1000.0;
  } else {
    *dens = 1.205 * exp(-z / 12e3);
    *tob = uz > eps ? (H - z) / uz : uz < -eps ? (thick - z) / uz : 1000.0;
  }
}
__device__ __forceinline__ void boundary(F2 z, F2 thick, F2 H, bool in_air, float uz, float rho,
                                         float* tob, float* dens) {
  const float eps = float(kEps64);
  float ahead = !in_air ? (uz > eps ? alt_sub(thick, z) : -(z.h + z.l))
                        : (uz > eps ? alt_sub(H, z) : alt_sub(thick, z));
  *tob = (uz > eps || uz < -eps) ? ahead / uz : 1000.f;
  *dens = !in_air ? rho : 1.205f * expf(-(z.h + z.l) * (1.f / 12e3f));
}

// The same with the porous top layer (src/Geometry.jl:617-635): the layer's
// lower face at pz is a boundary in both directions.
__device__ __forceinline__ void boundary_porous(double z, double thick, double H, double pz,
                                                bool in_air, bool in_p, double uz, double rho,
                                                double prho, double* tob, double* dens) {
  const double eps = kEps64;
  if (!in_air) {
    *dens = in_p ? prho : rho;
    const double next = z < pz ? pz : thick, prev = in_p ? pz : 0.0;
    *tob = uz > eps ? (next - z) / uz : uz < -eps ? (prev - z) / uz : 1000.0;
  } else {
    *dens = 1.205 * exp(-z / 12e3);
    *tob = uz > eps ? (H - z) / uz : uz < -eps ? (thick - z) / uz : 1000.0;
  }
}
__device__ __forceinline__ void boundary_porous(F2 z, F2 thick, F2 H, F2 pz, bool in_air,
                                                bool in_p, float uz, float rho, float prho,
                                                float* tob, float* dens) {
  const float eps = float(kEps64);
  float ahead;
  if (!in_air)
    ahead = uz > eps ? (in_p ? alt_sub(thick, z) : alt_sub(pz, z))
                     : (in_p ? alt_sub(pz, z) : -(z.h + z.l));
  else
    ahead = uz > eps ? alt_sub(H, z) : alt_sub(thick, z);
  *tob = (uz > eps || uz < -eps) ? ahead / uz : 1000.f;
  *dens = !in_air ? (in_p ? prho : rho) : 1.205f * expf(-(z.h + z.l) * (1.f / 12e3f));
}

// Advances a history by one transport step: ADV_STEP, ADV_DONE when it has
// ended, ADV_WAIT when the step suspended on a hard-event DCS sum,
// ADV_HANDOFF when phase 0 reached the mode switch.  H is Hist<R>, or
// HistP<R> for the geometry with the porous layer (medium 2: *porous).
template <class R, bool COOP, int PHASE, class H>
__device__ __forceinline__ int advance(const Med<R>& rock, const Med<R>& air, const Med<R>* porous,
                                       const Consts& C, H& h, Stream& g) {
  constexpr bool POR = std::is_same<H, HistP<R>>::value;
  const double eps = kEps64;
  State<R>& s = h.s;
  // FP32: thresholds are exactly representable (the host rounds them), eps
  // below their resolution
  const R thr = sizeof(R) == 8 ? R(C.thr) : R(C.thr_f);
  const R thr_low = sizeof(R) == 8 ? R(C.thr_low) : R(C.thr_low_f);
  for (int guard = 0; guard < 4; ++guard) {
    if (h.need_mode) {
      if (sizeof(R) == 8 ? !(double(s.E) < C.thr - eps) : !(s.E < thr)) return ADV_DONE;
      if (h.outer >= 1000) {
        s.status |= ST_OUTER_CAP;
        return ADV_DONE;
      }
      if (outside(s.z, h.H)) return ADV_DONE;
      if (!(s.w > R(0)) || !isfinite(s.w)) return ADV_DONE;
      if (sizeof(R) == 8 ? double(s.E) < C.thr_low - eps : s.E < thr_low) {
        if (PHASE == 1) {  // not reached: the energy never decreases
          s.status |= ST_OUTER_CAP;
          return ADV_DONE;
        }
        h.strag = C.straggling != 0;
        h.mixed = false;
        h.scat = C.scattering != 0;
        h.limit = fmin(thr_low, thr);
      } else {
        if (PHASE == 0) return ADV_HANDOFF;  // need_mode stays set for phase 1
        h.strag = false;
        h.mixed = C.straggling != 0;
        h.scat = false;
        h.limit = thr;
      }
      h.inner = 0;
      ++h.outer;
      h.need_mode = false;
    }
    const bool at_limit = sizeof(R) == 8 ? double(s.E) >= double(h.limit) - eps : s.E >= h.limit;
    if (h.inner >= 50000 || outside(s.z, h.H) || at_limit || !(s.w > R(0)) || !isfinite(s.w)) {
      h.need_mode = true;
      continue;
    }
    // medium, boundary distance and step (src/Geometry.jl:603-650, :461-476)
    const bool in_air = in_air_at(s.z, h.thick);
    int med = in_air ? 1 : 0;
    R tob, rd;
    const R uz = -s.uz;
    if constexpr (POR) {
      const bool in_p = !in_air && in_air_at(s.z, h.pz);  // z >= pz
      if (in_p) med = 2;
      boundary_porous(s.z, h.thick, h.H, h.pz, in_air, in_p, uz, h.rho, h.prho, &tob, &rd);
    } else {
      boundary(s.z, h.thick, h.H, in_air, uz, h.rho, &tob, &rd);
    }
    const Med<R>& m = med == 0 ? rock : (POR && med == 2 ? *porous : air);
    Loc<R> Li = locate(m, s.E);
    R Xi = at(m, Li, MC_CR);
    R lim = R(0.01) * Xi / fmax(rd, R(1e-6));
    // transport path at the start: the scattering step limit, then the soft
    // scattering of the step
    const R lb0 = h.scat ? transport_path(m, Li) : R(0);
    if (h.scat) {
      const R lb1 = lb0;
      if (lb1 > R(0) && rd > R(0)) lim = fmin(lim, R(0.01) * lb1 / rd);
    }
    if (in_air) lim = fmin(lim, R(0.05 * 12e3) / fmax(fabs(uz), R(0.05)));
    R step = fmin(tob + R(1e-7), lim);
    step = fmin(fmax(step, R(kStepMin)), R(1000));
    if (PHASE == 0 && h.strag) {
      if constexpr (PHASE == 0) {
        if (straggled_step<R, COOP>(m, C, s, Li, lb0, rd, step, g, h.scat, h.limit, h.x)) {
          h.x.kind = CONT_STRAG;
          h.x.medium = med;
          return ADV_WAIT;
        }
      }
    } else if (PHASE == 1 && h.mixed) {
      if constexpr (PHASE == 1) {
        if (mixed_step<R, COOP, true>(m, C, s, rd, step, g, h.limit, h.x)) {
          h.x.kind = CONT_MIXED;
          h.x.medium = med;
          return ADV_WAIT;
        }
      }
    } else {
      csda_step(m, C, s, Li, rd, step);
    }
    return step_done(h, C);
  }
  // The mode checks alternate without a step only if the thresholds were not
  // representable in R (the host rounds them); end the history flagged.
  s.status |= ST_OUTER_CAP;
  return ADV_DONE;
}

// Resumes a suspended step once h.x.total (and h.x.pick) hold the DCS sum.
template <class R, int PHASE, class H>
__device__ int resume(const Med<R>& rock, const Med<R>& air, const Med<R>* porous,
                      const Consts& C, H& h, Stream& g) {
  constexpr bool POR = std::is_same<H, HistP<R>>::value;
  Cont<R>& x = h.x;
  const Med<R>& m = x.medium == 0 ? rock : (POR && x.medium == 2 ? *porous : air);
  x.kind = CONT_NONE;
  const DelOutT<R> d = del_end(x.anc, x.denom, x.total, x.pick);
  if constexpr (PHASE == 1) {
    const R Emax = m.kcol(K_E)[m.nk - 1];
    if (mixed_event(h.s, x, d)) {
      mixed_end(h.s, x, Emax, h.limit, false);
    } else {
      ++x.event;
      if (mixed_run_in<R, true>(m, C, h.s, x, g, h.limit)) {
        x.kind = CONT_MIXED;
        return ADV_WAIT;
      }
    }
  } else {
    Loc<R> Li = locate(m, x.r0);
    const R lb0 = x.flag ? transport_path(m, Li) : R(0);
    straggled_end(m, C, h.s, Li, lb0, x.r0, d.energy, x.r1, x.r2, d.weight, d.process, d.element,
                  true, false, R(0), x.r3, x.a, true, x.flag != 0, g);
  }
  return step_done(h, C);
}

// A history handed from phase 0 to phase 1: its state, geometry, loop
// counters and random stream position.
template <class R>
struct Handoff {
  Alt<R> z, thick, H;
  R rho, ux, uy, uz, E, w;
  int status, steps, outer, used;
  uint32_t block, w0, w1, w2, w3;
  long index;       // history index (output slot)
  uint64_t stream;  // stream id
};
// The same with the porous layer of the history's column.
template <class R>
struct HandoffP : Handoff<R> {
  Alt<R> pz;
  R prho;
};
template <class R>
__device__ __forceinline__ void save_handoff(const Hist<R>& h, const Stream& g, long i,
                                             Handoff<R>* o) {
  Handoff<R> v;
  v.z = h.s.z;
  v.thick = h.thick;
  v.rho = h.rho;
  v.H = h.H;
  v.ux = h.s.ux;
  v.uy = h.s.uy;
  v.uz = h.s.uz;
  v.E = h.s.E;
  v.w = h.s.w;
  v.status = h.s.status;
  v.steps = h.steps;
  v.outer = h.outer;
  v.used = g.used;
  v.block = g.block;
  v.w0 = g.w0;
  v.w1 = g.w1;
  v.w2 = g.w2;
  v.w3 = g.w3;
  v.index = i;
  v.stream = uint64_t(g.c0) | (uint64_t(g.c1) << 32);
  *o = v;
}
template <class R>
__device__ __forceinline__ long load_handoff(const Handoff<R>& v, uint64_t seed, Hist<R>& h,
                                             Stream& g) {
  h.s.z = v.z;
  h.thick = v.thick;
  h.rho = v.rho;
  h.H = v.H;
  h.s.ux = v.ux;
  h.s.uy = v.uy;
  h.s.uz = v.uz;
  h.s.E = v.E;
  h.s.w = v.w;
  h.s.status = v.status;
  h.steps = v.steps;
  h.outer = v.outer;
  h.inner = 0;
  h.limit = R(0);
  h.need_mode = true;
  h.strag = h.mixed = h.scat = false;
  h.x.kind = CONT_NONE;
  g.init(seed, v.stream);
  g.block = v.block;
  g.used = v.used;
  g.w0 = v.w0;
  g.w1 = v.w1;
  g.w2 = v.w2;
  g.w3 = v.w3;
  return v.index;
}

// Porous layer of a history's column (HistP), written by the init kernel.
template <class R>
struct PorousRec {
  Alt<R> pz;
  R prho;
};
// Start record of a history, written by the init kernel in one converged
// pass (energy, charge and geometry draws, direction), read by phase 0.
template <class R>
struct StartRec {
  Alt<R> thick, H;
  double q, ws;  // charge and sampling weight (read back by the finish kernel)
  R E, rho, ux, uz;
};
// End record of a history, written by the transport, turned into the flux
// contribution by the finish kernel.
template <class R>
struct EndRec {
  Alt<R> z;
  R E, w, uz;
  int status, steps;
};

// Contribution of an ended history (src/Geometry.jl:729-757), FP64.
template <class R>
__device__ __forceinline__ double history_flux(const Consts& C, const EndRec<R>& e, double H,
                                               double q) {
  if (e.status & ST_FATAL) return 0.0;
  if (alt_value(e.z) >= H - 1.0 && double(e.E) < C.thr) {
    double c = fmin(fmax(-double(e.uz), 0.0), 1.0);
    if (c <= 0.0) return 0.0;
    double cs = cos_theta_star(c);
    return double(e.w) * gccly_flux(cs, pow(cs, 1.29), double(e.E), q, nullptr);
  }
  return 0.0;
}

}  // namespace mc
}  // namespace dp

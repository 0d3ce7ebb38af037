// common.cuh -- shared device/host helpers of libdpgpu: constants, the
// device table view, interval search, interpolation with tangents, Philox,
// bulk-copy (TMA) staging of table columns into shared memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/dpgpu.h"

#define DP_HD __host__ __device__ __forceinline__

namespace dp {

// Threads of the block that reduces one large CSC bucket (cells next to a
// detector hold thousands of entries).
constexpr int kBigThreads = 128;
// Sum over the kBigThreads threads of a block in a fixed order (shuffle tree
// per warp, then the warp partials in warp order); valid in thread 0.
__device__ __forceinline__ double big_block_sum(double v, double* sh /* kBigThreads / 32 */) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBigThreads / 32; ++w) s += sh[w];
  return s;
}

// src/Constants.jl:17-92 (values the path uses)
constexpr double kMuonMass = 0.10565839;
constexpr double kMuonCTau = 658.654;
constexpr double kElectronMass = 0.510998910e-3;
constexpr double kElectronRadius = 2.817940285e-15;
constexpr double kAlpha = 7.2973525693e-3;
constexpr double kHbarC = 1.973269804e-16;
constexpr double kBohrRadius = 0.529177210903e-10;
constexpr double kProtonMass = 0.938272;
constexpr double kNeutronMass = 0.939565;
constexpr double kPionMass = 0.13957018;
constexpr double kAvogadro = 6.02214076e23;
constexpr double kLarmor = 0.299792458;
constexpr double kPi = 3.14159265358979323846;
constexpr double kEps64 = 2.220446049250313e-16;
constexpr double kStepMin = 1e-7;

// Columns are padded to a multiple of 2 doubles so every column starts on a
// 16-byte boundary (required by cp.async.bulk).
DP_HD int padded(int n) { return (n + 1) & ~1; }

// Read-only view of the device tables: base[(mat * DP_NCOL + col) * ld + i].
struct TabView {
  const double* base;
  int n;        // energy nodes
  int ld;       // padded column stride
  int n_mat;
  int uniform;  // 1 if the log-energy grid is uniform
  double lE0, inv_dlE;
  DP_HD const double* col(int mat, int c) const { return base + ((size_t)mat * DP_NCOL + c) * ld; }
};

// Single-precision derived table columns (one row per energy node i; the
// per-interval columns hold the value of interval [i, i+1]):
//   RH, RL   range as a float pair (RH + RL = R to ~2^-48)
//   S        stopping power
//   E        kinetic energy
//   LE       log E
//   SLOPE    (logE[i+1]-logE[i]) / (R[i+1]-R[i])     (d log E / d R)
//   DSDLE    (S[i+1]-S[i]) / (logE[i+1]-logE[i])     (d S / d log E)
//   DLE      logE[i+1]-logE[i]
enum Col32 { C32_RH = 0, C32_RL, C32_S, C32_E, C32_LE, C32_SLOPE, C32_DSDLE, C32_DLE, kNC32 };
DP_HD int padded32(int n) { return (n + 3) & ~3; }

// ------------------------------------------------------------- dual numbers
// Value and tangent with respect to one scalar input (forward-mode AD).
struct Dd {
  double v, d;
};
DP_HD Dd dd(double v, double d = 0.0) { return Dd{v, d}; }
DP_HD Dd operator+(Dd a, Dd b) { return Dd{a.v + b.v, a.d + b.d}; }
DP_HD Dd operator-(Dd a, Dd b) { return Dd{a.v - b.v, a.d - b.d}; }
DP_HD Dd operator-(Dd a) { return Dd{-a.v, -a.d}; }
DP_HD Dd operator*(Dd a, Dd b) { return Dd{a.v * b.v, a.d * b.v + a.v * b.d}; }
DP_HD Dd operator*(double a, Dd b) { return Dd{a * b.v, a * b.d}; }
DP_HD Dd operator*(Dd a, double b) { return Dd{a.v * b, a.d * b}; }
DP_HD Dd operator/(Dd a, Dd b) {
  double q = a.v / b.v;
  return Dd{q, (a.d - q * b.d) / b.v};
}
DP_HD Dd operator/(Dd a, double b) { return Dd{a.v / b, a.d / b}; }
DP_HD Dd dexp(Dd a) {
  double e = exp(a.v);
  return Dd{e, e * a.d};
}
DP_HD Dd dlog(Dd a) { return Dd{log(a.v), a.d / a.v}; }
DP_HD Dd dsqrt(Dd a) {
  double s = sqrt(a.v);
  return Dd{s, a.d / (2.0 * s)};
}
DP_HD Dd dmin(Dd a, Dd b) { return (b.v < a.v) ? b : a; }
DP_HD Dd dmax(Dd a, Dd b) { return (b.v > a.v) ? b : a; }

// ------------------------------------------------------------- interval search
// Largest i in [0, n-2] with xs[i] <= x, the interval a bisection of
// src/Physics.jl:672-680 selects for x inside (xs[0], xs[n-1]).
DP_HD int bisect(const double* xs, int n, double x) {
  int lo = 0, hi = n - 1;
  while (lo < hi - 1) {
    int mid = (lo + hi) >> 1;
    if (x < xs[mid]) hi = mid; else lo = mid;
  }
  return lo;
}
// Same interval starting from a hint known to be <= the answer (monotone walks).
DP_HD int walk_up(const double* xs, int n, double x, int hint) {
  int i = hint < 0 ? 0 : hint;
  if (i > n - 2) i = n - 2;
  while (i > 0 && x < xs[i]) --i;
  while (i < n - 2 && !(x < xs[i + 1])) ++i;
  return i;
}
// O(1) interval on a uniform log grid, corrected to the bisection answer.
DP_HD int uniform_interval(const double* lxs, int n, double lx, double lE0, double inv_d) {
  double f = floor((lx - lE0) * inv_d);
  int i = f < 0.0 ? 0 : (f > double(n - 2) ? n - 2 : int(f));
  while (i > 0 && lx < lxs[i]) --i;
  while (i < n - 2 && !(lx < lxs[i + 1])) ++i;
  return i;
}

// Property lookup y(E) linear in log E, clamped at the ends, with the
// derivative carried through log E only (src/Physics.jl:660-687 and the rrule
// at :716-739).  E is a dual; logE = log(E) supplied by the caller.
DP_HD Dd interp_logE(const TabView& t, const double* xs, const double* lxs, const double* ys,
                     Dd E, Dd logE, int* hint) {
  int n = t.n;
  if (E.v <= xs[0]) return dd(ys[0]);
  if (E.v >= xs[n - 1]) return dd(ys[n - 1]);
  int i = t.uniform ? uniform_interval(lxs, n, logE.v, t.lE0, t.inv_dlE)
                    : (hint ? walk_up(lxs, n, logE.v, *hint) : bisect(lxs, n, logE.v));
  if (hint) *hint = i;
  double s = (ys[i + 1] - ys[i]) / (lxs[i + 1] - lxs[i]);
  double tt = (logE.v - lxs[i]) / (lxs[i + 1] - lxs[i]);
  return Dd{ys[i] + tt * (ys[i + 1] - ys[i]), s * logE.d};
}
// Inverse range (src/Physics.jl:833-867): E(X) = exp(log-linear in X).
DP_HD Dd inverse_range(const double* R, const double* E, const double* lE, int n, Dd X,
                       int* hint) {
  if (X.v <= R[0]) return dd(E[0]);
  if (X.v >= R[n - 1]) return dd(E[n - 1]);
  int i = hint ? walk_up(R, n, X.v, *hint) : bisect(R, n, X.v);
  if (hint) *hint = i;
  double tt = (X.v - R[i]) / (R[i + 1] - R[i]);
  double le = lE[i] + tt * (lE[i + 1] - lE[i]);
  double e = exp(le);
  return Dd{e, e * (lE[i + 1] - lE[i]) / (R[i + 1] - R[i]) * X.d};
}

// ------------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon et al. (SC'11): 10 rounds, Weyl key bumps.
struct U4 {
  uint32_t x, y, z, w;
};
DP_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return uint32_t((uint64_t(a) * uint64_t(b)) >> 32);
#endif
}
DP_HD U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t h0 = mulhi32(0xD2511F53u, c.x), l0 = 0xD2511F53u * c.x;
    uint32_t h1 = mulhi32(0xCD9E8D57u, c.z), l1 = 0xCD9E8D57u * c.z;
    c = U4{h1 ^ c.y ^ k0, l1, h0 ^ c.w ^ k1, l0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}
// Uniform double in [0, 1) from two 32-bit words (53 random bits).
DP_HD double u01(uint32_t a, uint32_t b) {
  return (double(a >> 5) * 67108864.0 + double(b >> 6)) * (1.0 / 9007199254740992.0);
}

// run_backward_mc sample i (src/Geometry.jl:863-875): log-uniform energy and
// +-1 charge from one Philox block keyed by (seed, i); stream word 0.
DP_HD void mc_sample(uint64_t seed, uint64_t i, double emin, double emax, double* E, double* q,
                     double* w) {
  U4 r = philox(U4{uint32_t(i), uint32_t(i >> 32), 0u, 0u}, uint32_t(seed), uint32_t(seed >> 32));
  double rk = log(emax / emin);
  double u1 = u01(r.x, r.y), u2 = u01(r.z, r.w);
  double kf, wf;
  if (rk > 0.0) {
    kf = emin * exp(rk * u1);
    wf = kf * rk;
  } else {
    kf = emin;
    wf = 1.0;
  }
  *E = kf;
  *q = u2 > 0.5 ? 1.0 : -1.0;
  *w = wf * 2.0;
}

// ------------------------------------------------------------- GCCLY flux
// src/GaisserFlux.jl:62-76
DP_HD double cos_theta_star(double c) {
  const double p0 = 0.102573, p1 = -0.068287, p2 = 0.958633, p3 = 0.0407253, p4 = 0.817285;
  double cs2 = (c * c + p0 * p0 + p1 * pow(c, p2) + p3 * pow(c, p4)) / (1.0 + p0 * p0 + p1 + p3);
  return cs2 > 0.0 ? sqrt(cs2) : 0.0;
}
DP_HD double charge_fraction(double q) {
  const double r = 1.2766;
  return q < 0.0 ? 1.0 / (1.0 + r) : (q > 0.0 ? r / (1.0 + r) : 1.0);
}
// flux_gccly (src/GaisserFlux.jl:125-133, :93-105) with cos_theta_star(c) and
// cs^1.29 precomputed by the caller (they depend on the direction only).
// Returns the flux; *dlog receives d log(flux)/dK.
DP_HD double gccly_flux(double cs, double cs129, double K, double q, double* dlog) {
  double Emu = K + kMuonMass;
  double a = 3.64 / (Emu * cs129);
  double g = pow(1.0 + a, -2.7);
  double ec = 1.1 * Emu * cs;
  double rpi = 1.0 + ec / 115.0, rK = 1.0 + ec / 850.0;
  double h = 1.0 / rpi + 0.054 / rK;
  double f = g * (1.4e3 * pow(Emu, -2.7) * h * charge_fraction(q));
  if (dlog) {
    double dh = -(1.1 * cs / 115.0) / (rpi * rpi) - 0.054 * (1.1 * cs / 850.0) / (rK * rK);
    *dlog = -2.7 * (-a / Emu) / (1.0 + a) - 2.7 / Emu + dh / h;
  }
  return f;
}

// ------------------------------------------------------------- altitude pairs
// An unevaluated pair hi + lo of floats (about 48 bits) for positions in the
// FP32 transports: compensated updates and differences, no FP64 instruction.
struct F2 {
  float h, l;
};
DP_HD F2 f2_make(double v) {
  float h = float(v);
  return F2{h, float(v - double(h))};
}
// z += dz (TwoSum of the high parts, error folded into the low part)
DP_HD void alt_add(F2& z, float dz) {
  float s = z.h + dz, bp = s - z.h;
  float e = (z.h - (s - bp)) + (dz - bp);
  float l = z.l + e, h = s + l;
  z.l = l - (h - s);
  z.h = h;
}
// a - b as a float
DP_HD float alt_sub(F2 a, F2 b) { return (a.h - b.h) + (a.l - b.l); }

// ------------------------------------------------------------- tallies
// Compensated (TwoSum) accumulator for the deterministic FP64 tallies.
struct KSum {
  double s, c;
};
DP_HD void kadd(KSum& a, double x) {
  double t = a.s + x;
  double bp = t - a.s;
  a.c += (a.s - (t - bp)) + (x - bp);
  a.s = t;
}
DP_HD void kmerge(KSum& a, const KSum& b) {
  kadd(a, b.s);
  a.c += b.c;
}

// ------------------------------------------------------------- staging (TMA)
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return uint32_t(__cvta_generic_to_shared(p));
}
// Iteration limit of a staging wait (mbarrier try_wait polls).  A context can
// lower the first wait's limit for failure-path tests (dp_set_debug_limits);
// the wait for copies still in flight always uses this one.
constexpr int kStageWait = 1 << 22;

__device__ __forceinline__ bool mbar_wait(uint32_t bar, int iters) {
  uint32_t done = 0;
  for (int it = 0; it < iters && !done; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(0)
        : "memory");
  }
  return done != 0;
}
// Ends a staging wait of the whole block: true when every thread saw the
// copies land.  Otherwise the threads whose wait gave up wait once more
// (bounded) for the copies in flight, so that no bulk copy still writes this
// block's shared memory when it leaves, and the result is false.
__device__ __forceinline__ bool stage_settle(uint32_t bar, bool done) {
  if (__syncthreads_and(done) != 0) return true;
  if (!done) mbar_wait(bar, kStageWait);
  return false;
}
__device__ __forceinline__ void mbar_init(uint32_t bar) {
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
}
// Copies `ncol` columns of `bytes` bytes each (16-byte multiples, 16-byte
// aligned) from global to shared memory with cp.async.bulk completing on one
// mbarrier.  All threads of the block call it.  Returns false if the wait
// exceeded `wait_iters` polls (the copies have then landed or their own
// bounded wait gave up too; the block must skip its work).
__device__ __forceinline__ bool stage_columns(double* smem_dst, const double* const* src, int ncol,
                                              uint32_t bytes, uint64_t* mbar,
                                              int wait_iters = kStageWait) {
  uint32_t bar = smem_u32(mbar);
  mbar_init(bar);
  if (threadIdx.x == 0) {
    uint32_t total = bytes * uint32_t(ncol);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(total)
                 : "memory");
    for (int c = 0; c < ncol; ++c) {
      uint32_t dst = smem_u32(smem_dst + size_t(c) * (bytes / 8));
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              dst),
          "l"(src[c]), "r"(bytes), "r"(bar)
          : "memory");
    }
  }
  return stage_settle(bar, mbar_wait(bar, wait_iters));
}
#endif

}  // namespace dp

// csda_mc.cu -- backward Monte Carlo in CSDA mode (run_backward_mc with
// straggling = scattering = false) and its density derivative.
//
// One thread per history.  The history follows the adaptive two-layer step
// sequence of src/Geometry.jl:534-672 (transport_backward_step :424-457,
// step limit :461-476) and the acceptance of :694-757.  The derivative with
// respect to the rock density is propagated in tangent (forward) mode through
// the same discrete program: for a single scalar density this is the cheapest
// exact adjoint and equals what Zygote computes on the reference
// (compute_flux_gradient, :1007-1028), step-size dependence on rho included.
//
// Tables used by a history (energy grid and the rock/air CSDA range and
// stopping power) are staged once per CTA into shared memory with
// cp.async.bulk.  Per-history results go to global memory and are reduced in a
// fixed order (compensated), so estimates are bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace dp {

// Geometry of one history: the two-layer column and the direction-dependent
// constants of the acceptance flux.
struct CsdaGeo {
  double thickness, rho, H, dir_z, uz, air_limit, cos_final, cs, cs129;
};
__host__ __device__ inline CsdaGeo csda_geo(double thickness, double rho, double elevation, double H) {
  CsdaGeo g;
  double theta = (90.0 - elevation) * kPi / 180.0;
  double c = cos(theta);
  g.thickness = thickness;
  g.rho = rho;
  g.H = H;
  g.dir_z = -c;
  g.uz = c;
  g.air_limit = 0.05 * 12e3 / fmax(fabs(c), 0.05);
  g.cos_final = fmin(fmax(c, 0.0), 1.0);
  g.cs = cos_theta_star(g.cos_final);
  g.cs129 = pow(g.cs, 1.29);
  return g;
}

struct CsdaParams {
  TabView tab;
  int rock, air;
  CsdaGeo geo;  // fixed geometry (los == nullptr)
  double threshold, low, mass, ctau;
  int use_philox;
  uint64_t seed;
  double emin, emax;
  long n;
  const double *E, *q, *w;
  double *contrib, *dcontrib, *sample_out;
  int32_t* steps;
  int* err_flag;  // 1: a table-staging wait gave up; 4: a history reached step_cap
  int step_cap, wait_iters;
  // lines of sight: history i belongs to the record l with
  // los_off[l] <= i < los_off[l + 1] and takes its geometry and energy range
  const dp_los* los;
  const int64_t* los_off;
  long n_los;
};

// Shared-memory table slots (all materials share the energy grid): the six
// staged columns, then per-interval columns derived from them once per block
// (1 / (R[i+1] - R[i]) and S[i+1] - S[i] per material, log-energy widths).
enum { S_E = 0, S_LOGE, S_RS, S_RR, S_AS, S_AR, S_NCOL };
enum { D_RINV = 0, D_RDS, D_AINV, D_ADS, D_DLE, D_NCOL };
constexpr int kCsdaThreads = 64;

// d(a^-1/2) = -1/2 a^-3/2 da
__device__ __forceinline__ Dd drsqrt(Dd a) {
  double r = rsqrt(a.v);
  return Dd{r, -0.5 * r * r * r * a.d};
}

// One material's columns as one history walks them.
struct CsdaMat {
  const double *R, *S, *rinv, *ds;
};

// The CSDA history loop of run_backward_mc (src/Geometry.jl:534-672 with
// transport_backward_step, :424-457, and the step limit, :461-476), in FP64
// with the density tangent, arranged so that one step costs one exp and one
// rsqrt:
//  - the range at the end of a step is carried into the next step (the
//    reference recomputes it from the energy: R(K(Y)) = Y to rounding);
//  - the inverse range locates Y's interval and gives log E' = logE[i] +
//    t dlogE[i] without a log, and S(E') = S[i] + t dS[i] on the same
//    interval and parameter (the reference interpolates S at log(E'), the
//    same point to rounding);
//  - the stopping-power ratios S(E')/S(E) of consecutive steps in one
//    material telescope to S(end)/S(start) of the material's run, and the
//    decay factors multiply to exp(-sum dt / c tau);
//  - beta gamma = sqrt(gamma^2 - 1) with gamma the mean of the step's end
//    points, so dt = step * rsqrt(gamma^2 - 1).
// Every branch the reference takes (boundaries, step limits and clamps, the
// energy ceiling, the acceptance) is the same, and the results agree with
// the reference's operation-by-operation program to rounding (~1e-13).
__global__ void __launch_bounds__(kCsdaThreads) csda_mc_kernel(CsdaParams P) {
  extern __shared__ __align__(16) double smem[];
  __shared__ uint64_t mbar;
  const int ld = P.tab.ld, n = P.tab.n;
  const double* src[S_NCOL] = {P.tab.col(0, DP_COL_E),          P.tab.col(0, DP_COL_LOGE),
                               P.tab.col(P.rock, DP_COL_CSDA_S), P.tab.col(P.rock, DP_COL_CSDA_R),
                               P.tab.col(P.air, DP_COL_CSDA_S),  P.tab.col(P.air, DP_COL_CSDA_R)};
  if (!stage_columns(smem, src, S_NCOL, uint32_t(ld * sizeof(double)), &mbar, P.wait_iters)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    return;
  }
  const double* sE = smem + S_E * ld;
  const double* slE = smem + S_LOGE * ld;
  double* der = smem + S_NCOL * ld;
  for (int k = threadIdx.x; k < n - 1; k += blockDim.x) {
    const double* rR = smem + S_RR * ld;
    const double* rS = smem + S_RS * ld;
    const double* aR = smem + S_AR * ld;
    const double* aS = smem + S_AS * ld;
    der[D_RINV * ld + k] = 1.0 / (rR[k + 1] - rR[k]);
    der[D_RDS * ld + k] = rS[k + 1] - rS[k];
    der[D_AINV * ld + k] = 1.0 / (aR[k + 1] - aR[k]);
    der[D_ADS * ld + k] = aS[k + 1] - aS[k];
    der[D_DLE * ld + k] = slE[k + 1] - slE[k];
  }
  __syncthreads();
  const CsdaMat rockM{smem + S_RR * ld, smem + S_RS * ld, der + D_RINV * ld, der + D_RDS * ld};
  const CsdaMat airM{smem + S_AR * ld, smem + S_AS * ld, der + D_AINV * ld, der + D_ADS * ld};
  const double* dle = der + D_DLE * ld;
  const double eps = kEps64;
  const double half_inv_m = 0.5 / P.mass;
  const int32_t cap = P.step_cap;
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < P.n;
       i += long(gridDim.x) * blockDim.x) {
    double E0, q, w;
    CsdaGeo G = P.geo;
    if (P.los) {
      long lo = 0, hi = P.n_los;
      while (hi - lo > 1) {
        long mid = (lo + hi) >> 1;
        if (P.los_off[mid] <= i) lo = mid; else hi = mid;
      }
      const dp_los& L = P.los[lo];
      double H = L.air_height > 0.0 ? L.thickness + L.air_height
                                    : (L.primary_altitude > 0.0 ? L.primary_altitude : 3e4);
      G = csda_geo(L.thickness, L.density, L.elevation, H);
      mc_sample(P.seed, uint64_t(i), L.energy_min,
                L.energy_max > L.energy_min ? L.energy_max : L.energy_min, &E0, &q, &w);
    } else if (P.use_philox) {
      mc_sample(P.seed, uint64_t(i), P.emin, P.emax, &E0, &q, &w);
      if (P.sample_out) {
        P.sample_out[3 * i] = E0;
        P.sample_out[3 * i + 1] = q;
        P.sample_out[3 * i + 2] = w;
      }
    } else {
      E0 = P.E[i];
      q = P.q[i];
      w = P.w[i];
    }
    const Dd rho = dd(G.rho, 1.0);
    const Dd c_rock = dd(0.01, 0.0) / dmax(rho, dd(1e-6));  // 0.01 / rho
    const double inv_uz = G.uz > eps || G.uz < -eps ? 1.0 / G.uz : 0.0;
    Dd E = dd(E0), lE = dd(log(E0)), z = dd(0.0), tau = dd(0.0);
    Dd wS = dd(1.0), Sstart = dd(1.0), Scur = dd(1.0), X = dd(0.0);
    int mat = -1, k = 0;
    int32_t nsteps = 0;
    while (nsteps < cap) {
      if (!(E.v < P.threshold - eps)) break;
      if (z.v < 0.0 || z.v >= G.H - eps) break;
      const int m = z.v >= G.thickness ? 1 : 0;
      const CsdaMat M = m ? airM : rockM;
      if (m != mat) {
        // entering a material: range and stopping power at E from the
        // log-energy interpolation (src/Physics.jl:660-687), as the
        // reference's first step in it does
        if (mat >= 0) wS = wS * (Scur / Sstart);
        mat = m;
        X = interp_logE(P.tab, sE, slE, M.R, E, lE, nullptr);
        Sstart = interp_logE(P.tab, sE, slE, M.S, E, lE, nullptr);
        Scur = Sstart;
        k = E.v <= sE[0] ? 0 : (E.v >= sE[n - 1] ? n - 2
                                                  : uniform_interval(slE, n, lE.v, P.tab.lE0,
                                                                     P.tab.inv_dlE));
      }
      Dd dens, tob, lim;
      if (m == 0) {
        dens = rho;
        if (G.uz > eps) tob = (dd(G.thickness) - z) * inv_uz;
        else if (G.uz < -eps) tob = (dd(0.0) - z) * inv_uz;
        else tob = dd(1000.0);
        lim = X * c_rock;
      } else {
        dens = 1.205 * dexp(z / -12e3);
        if (G.uz > eps) tob = (dd(G.H) - z) * inv_uz;
        else if (G.uz < -eps) tob = (dd(G.thickness) - z) * inv_uz;
        else tob = dd(1000.0);
        lim = dmin(0.01 * X / dmax(dens, dd(1e-6)), dd(G.air_limit));
      }
      Dd step = dmin(tob + dd(1e-7), lim);
      if (step.v < kStepMin) step = dd(kStepMin);
      else if (step.v > 1000.0) step = dd(1000.0);
      // inverse range at Y (src/Physics.jl:833-867), clamped at the table ends
      const Dd Y = X + step * dens;
      Dd Ef, lEf, Sf;
      if (Y.v <= M.R[0]) {
        k = 0;
        Ef = dd(sE[0]);
        lEf = dd(slE[0]);
        Sf = dd(M.S[0]);
      } else if (Y.v >= M.R[n - 1]) {
        k = n - 2;
        Ef = dd(sE[n - 1]);
        lEf = dd(slE[n - 1]);
        Sf = dd(M.S[n - 1]);
      } else {
        k = walk_up(M.R, n, Y.v, k);
        const Dd t = (Y - dd(M.R[k])) * M.rinv[k];
        lEf = dd(slE[k]) + t * dle[k];
        Ef = dexp(lEf);
        Sf = dd(M.S[k]) + t * M.ds[k];
      }
      // proper time of the step at the mean Lorentz factor
      const Dd ga = dd(1.0) + (E + Ef) * half_inv_m;
      const Dd g2 = ga * ga - dd(1.0);
      const Dd dt = g2.v > 1e-12 * ga.v * ga.v ? step * drsqrt(g2) : step / (1e-6 * ga);
      tau = tau + dt;
      z = z - step * dd(G.dir_z);
      X = Y;
      E = Ef;
      lE = lEf;
      Scur = Sf;
      ++nsteps;
    }
    if (mat >= 0) wS = wS * (Scur / Sstart);
    const Dd wt = wS * dexp(tau / -P.ctau);
    double f = 0.0, df = 0.0;
    if (nsteps >= cap) atomicExch(P.err_flag, 4);
    else if (z.v >= G.H - 1.0 && E.v < P.threshold && G.cos_final > 0.0) {
      double dlogf;
      double F = gccly_flux(G.cs, G.cs129, E.v, q, &dlogf);
      f = wt.v * F;
      df = wt.d * F + wt.v * F * dlogf * E.d;
    }
    P.contrib[i] = w * f;
    if (P.dcontrib) P.dcontrib[i] = w * df;
    if (P.steps) P.steps[i] = nsteps;
  }
}

// ------------------------------------------------------------ mixed precision
// The same history loop with the transport and its density tangent in FP32
// (the single-precision derived columns: range pairs, stopping power,
// energy, log energy and the per-interval slopes), the range, its tangent
// and the altitude as float pairs, FP64 only for the start offset, the final
// energy and the flux.  A history's flux and d flux / d rho stay within ~1e-6
// of the FP64 program: the FP64 pipe runs at 1/64 of the FP32 rate on this
// GPU, and a CSDA history is a chain of 10^2-10^3 dependent steps.
struct Df {
  float v, d;
};
__device__ __forceinline__ Df operator+(Df a, Df b) { return Df{a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Df operator-(Df a, Df b) { return Df{a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Df operator*(Df a, Df b) { return Df{a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Df operator*(float a, Df b) { return Df{a * b.v, a * b.d}; }
__device__ __forceinline__ Df operator/(Df a, Df b) {
  float q = a.v / b.v;
  return Df{q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Df fexp(Df a) {
  float e = expf(a.v);
  return Df{e, e * a.d};
}
__device__ __forceinline__ Df fsqrt(Df a) {
  float r = sqrtf(a.v);
  return Df{r, a.d / (2.f * r)};
}
__device__ __forceinline__ Df fmin2(Df a, Df b) { return b.v < a.v ? b : a; }
__device__ __forceinline__ Df fmax2(Df a, Df b) { return b.v > a.v ? b : a; }

// exp(x) - 1 for an offset inside one log-energy interval: its Taylor series
// to x^7 (truncation below 2e-9 relative for |x| <= 0.25), expm1f beyond.
__device__ __forceinline__ float expm1_small(float x) {
  if (fabsf(x) > 0.25f) return expm1f(x);
  return x * (1.f + x * (0.5f + x * (1.f / 6.f + x * (1.f / 24.f + x * (1.f / 120.f +
                                               x * (1.f / 720.f + x * (1.f / 5040.f)))))));
}

// Staged FP32 columns per material (rock, air); RL is the low part of the
// range pair.
enum { F_R = 0, F_RL, F_S, F_E, F_LE, F_SLOPE, F_DSDLE, F_DLE, F_NCOL };

struct Tab32 {
  const float *R, *RL, *S, *E, *LE, *SLOPE, *DSDLE, *DLE;
};
__device__ __forceinline__ int f_interval(const Tab32& t, int n, float lx, const TabView& tv) {
  int i;
  if (tv.uniform) {
    float f = floorf((lx - float(tv.lE0)) * float(tv.inv_dlE));
    i = !(f >= 0.f) ? 0 : (f > float(n - 2) ? n - 2 : int(f));
  } else {
    i = 0;
  }
  while (i > 0 && lx < t.LE[i]) --i;
  while (i < n - 2 && !(lx < t.LE[i + 1])) ++i;
  return i;
}

// The lean step of csda_mc_kernel in FP32: one exponential and one rsqrt per
// step, telescoped stopping-power ratios, a summed decay exponent.  What
// keeps a history within ~1e-6 of the FP64 program:
//  - the range and its density tangent are float pairs (TwoSum), so that
//    10^2-10^3 increments do not drift;
//  - the energy at a range is E_k (1 + expm1(dle)) with dle the log-energy
//    offset inside interval k (|dle| <= one grid step), not exp(log E_k +
//    dle): a float log E carries an absolute error of ~1e-6;
//  - the history's starting offset comes from (E0 - E_k) / E_k, and the
//    energy that enters the flux is formed in FP64 from the FP64 node E_k;
//  - a material entered mid-walk is located by the interval and offset the
//    walk already holds (all materials share the energy grid).
__global__ void __launch_bounds__(128) csda32_kernel(CsdaParams P, const float* tab32, int ld32) {
  extern __shared__ __align__(16) double smem[];
  __shared__ uint64_t mbar;
  const int n = P.tab.n;
  const int cols[F_NCOL] = {C32_RH, C32_RL, C32_S, C32_E, C32_LE, C32_SLOPE, C32_DSDLE, C32_DLE};
  // FP32 columns are staged as pairs of doubles: ld32 floats = ld32/2 doubles
  const double* src[2 * F_NCOL];
  for (int m = 0; m < 2; ++m)
    for (int c = 0; c < F_NCOL; ++c)
      src[m * F_NCOL + c] = reinterpret_cast<const double*>(
          tab32 + (size_t(m == 0 ? P.rock : P.air) * kNC32 + cols[c]) * ld32);
  if (!stage_columns(smem, src, 2 * F_NCOL, uint32_t(ld32 * sizeof(float)), &mbar, P.wait_iters)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    return;
  }
  const float* sf = reinterpret_cast<const float*>(smem);
  auto tab = [&](int m) {
    const float* b = sf + size_t(m) * F_NCOL * ld32;
    return Tab32{b + F_R * ld32,  b + F_RL * ld32,    b + F_S * ld32,     b + F_E * ld32,
                 b + F_LE * ld32, b + F_SLOPE * ld32, b + F_DSDLE * ld32, b + F_DLE * ld32};
  };
  const double* E64 = P.tab.col(0, DP_COL_E);
  const float mass = float(P.mass), ctau = float(P.ctau);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < P.n;
       i += long(gridDim.x) * blockDim.x) {
    double E0, q, w;
    CsdaGeo G = P.geo;
    if (P.los) {
      long lo = 0, hi = P.n_los;
      while (hi - lo > 1) {
        long mid = (lo + hi) >> 1;
        if (P.los_off[mid] <= i) lo = mid; else hi = mid;
      }
      const dp_los& L = P.los[lo];
      double H = L.air_height > 0.0 ? L.thickness + L.air_height
                                    : (L.primary_altitude > 0.0 ? L.primary_altitude : 3e4);
      G = csda_geo(L.thickness, L.density, L.elevation, H);
      mc_sample(P.seed, uint64_t(i), L.energy_min,
                L.energy_max > L.energy_min ? L.energy_max : L.energy_min, &E0, &q, &w);
    } else if (P.use_philox) {
      mc_sample(P.seed, uint64_t(i), P.emin, P.emax, &E0, &q, &w);
    } else {
      E0 = P.E[i];
      q = P.q[i];
      w = P.w[i];
    }
    const Df rho{float(G.rho), 1.f};
    const Df c_rock = Df{0.01f, 0.f} / fmax2(rho, Df{1e-6f, 0.f});
    const F2 thick = f2_make(G.thickness), Htop = f2_make(G.H);
    const float uz = float(G.uz), dir_z = float(G.dir_z), air_limit = float(G.air_limit);
    const float eps = float(kEps64);
    const float inv_uz = uz > eps || uz < -eps ? 1.f / uz : 0.f;
    const float thr = float(P.threshold), half_inv_m = 0.5f / mass;
    // position on the energy grid: interval k and offset dle (value and
    // tangent); edge -1 / +1: clamped at the first / last node
    int k, edge = 0;
    Df dle{0.f, 0.f};
    {
      const Tab32 t0 = tab(0);
      if (E0 <= E64[0]) {
        k = 0;
        edge = -1;
      } else if (E0 >= E64[n - 1]) {
        k = n - 2;
        edge = 1;
        dle.v = t0.DLE[n - 2];
      } else {
        k = f_interval(t0, n, logf(float(E0)), P.tab);
        while (k > 0 && E0 < E64[k]) --k;
        while (k < n - 2 && !(E0 < E64[k + 1])) ++k;
        dle.v = log1pf(float(E0 - E64[k]) / float(E64[k]));
      }
    }
    Df E{float(E0), 0.f}, tau{0.f, 0.f};
    Df wS{1.f, 0.f}, Sstart{1.f, 0.f}, Scur{1.f, 0.f};
    F2 X{0.f, 0.f}, Xd{0.f, 0.f}, z{0.f, 0.f};
    float zd = 0.f, em1 = 0.f;
    bool moved = false;
    int mat = -1;
    int32_t nsteps = 0;
    const int32_t cap = P.step_cap;
    while (nsteps < cap) {
      if (!(E.v < thr)) break;
      if (z.h + z.l < 0.f || alt_sub(z, Htop) >= 0.f) break;
      const int m = alt_sub(z, thick) >= 0.f ? 1 : 0;
      const Tab32 t = tab(m);
      if (m != mat) {
        // range and stopping power at the current energy, linear in log E on
        // interval k (src/Physics.jl:660-687), clamped at the ends
        if (mat >= 0) wS = wS * (Scur / Sstart);
        mat = m;
        if (edge != 0) {
          const int j = edge < 0 ? 0 : n - 1;
          X = F2{t.R[j], t.RL[j]};
          Xd = F2{0.f, 0.f};
          Sstart = Df{t.S[j], 0.f};
        } else {
          const float tt = dle.v / t.DLE[k];
          X = F2{t.R[k], t.RL[k]};
          alt_add(X, tt * ((t.R[k + 1] - t.R[k]) + (t.RL[k + 1] - t.RL[k])));
          Xd = F2{dle.d / t.SLOPE[k], 0.f};
          Sstart = Df{t.S[k] + dle.v * t.DSDLE[k], dle.d * t.DSDLE[k]};
        }
        Scur = Sstart;
      }
      Df dens, lim;
      float ahead;
      const Df Xv{X.h + X.l, Xd.h + Xd.l};
      if (m == 0) {
        dens = rho;
        ahead = uz > eps ? alt_sub(thick, z) : -(z.h + z.l);
        lim = Xv * c_rock;
      } else {
        const float dv = 1.205f * expf(-(z.h + z.l) * (1.f / 12e3f));
        dens = Df{dv, -dv / 12e3f * zd};
        ahead = uz > eps ? alt_sub(Htop, z) : alt_sub(thick, z);
        lim = fmin2(0.01f * Xv / fmax2(dens, Df{1e-6f, 0.f}), Df{air_limit, 0.f});
      }
      const Df tob = inv_uz != 0.f ? Df{ahead * inv_uz, -zd * inv_uz} : Df{1000.f, 0.f};
      Df step = tob.v + 1e-7f <= lim.v ? Df{tob.v + 1e-7f, tob.d} : lim;
      if (step.v < float(kStepMin)) step = Df{float(kStepMin), 0.f};
      else if (step.v > 1000.f) step = Df{1000.f, 0.f};
      // Y = X + step * dens (pairs), and the inverse range at Y
      // (src/Physics.jl:833-867)
      F2 Y = X, Yd = Xd;
      alt_add(Y, step.v * dens.v);
      alt_add(Yd, step.d * dens.v + step.v * dens.d);
      const float Yv = Y.h + Y.l;
      Df Ef, Sf;
      if (Yv <= t.R[0]) {
        k = 0;
        edge = -1;
        dle = Df{0.f, 0.f};
        Ef = Df{t.E[0], 0.f};
        Sf = Df{t.S[0], 0.f};
      } else if (Yv >= t.R[n - 1]) {
        k = n - 2;
        edge = 1;
        dle = Df{t.DLE[n - 2], 0.f};
        Ef = Df{t.E[n - 1], 0.f};
        Sf = Df{t.S[n - 1], 0.f};
      } else {
        while (k > 0 && Yv < t.R[k]) --k;
        while (k < n - 2 && !(Yv < t.R[k + 1])) ++k;
        edge = 0;
        dle = Df{alt_sub(Y, F2{t.R[k], t.RL[k]}) * t.SLOPE[k], (Yd.h + Yd.l) * t.SLOPE[k]};
        em1 = expm1_small(dle.v);
        const float ev = t.E[k] + t.E[k] * em1;
        Ef = Df{ev, ev * dle.d};
        Sf = Df{t.S[k] + dle.v * t.DSDLE[k], dle.d * t.DSDLE[k]};
      }
      // proper time of the step at the mean Lorentz factor
      const Df ga = Df{1.f, 0.f} + (E + Ef) * Df{half_inv_m, 0.f};
      const Df g2 = ga * ga - Df{1.f, 0.f};
      Df dt;
      if (g2.v > 1e-12f * ga.v * ga.v) {
        const float r = rsqrtf(g2.v);
        dt = step * Df{r, -0.5f * r * r * r * g2.d};
      } else {
        dt = step / (Df{1e-6f, 0.f} * ga);
      }
      tau = tau + dt;
      alt_add(z, -(step.v * dir_z));
      zd -= step.d * dir_z;
      X = Y;
      Xd = Yd;
      E = Ef;
      Scur = Sf;
      moved = true;
      ++nsteps;
    }
    if (mat >= 0) wS = wS * (Scur / Sstart);
    const Df wt = wS * fexp(Df{-1.f / ctau, 0.f} * tau);
    // the final energy in FP64 from the FP64 node
    const double Efin = !moved     ? E0
                        : edge < 0 ? E64[0]
                        : edge > 0 ? E64[n - 1]
                                   : E64[k] + E64[k] * double(em1);
    double f = 0.0, df = 0.0;
    if (nsteps >= cap) atomicExch(P.err_flag, 4);
    else if (alt_sub(z, Htop) >= -1.f && Efin < P.threshold && G.cos_final > 0.0) {
      double dlogf;
      double F = gccly_flux(G.cs, G.cs129, Efin, q, &dlogf);
      f = double(wt.v) * F;
      df = double(wt.d) * F + double(wt.v) * F * dlogf * double(E.d);
    }
    P.contrib[i] = w * f;
    if (P.dcontrib) P.dcontrib[i] = w * df;
    if (P.steps) P.steps[i] = nsteps;
  }
}

// Compensated (TwoSum) accumulation in a fixed order: every thread owns a
// fixed strided subset, blocks reduce in a fixed tree, a single block then
// reduces the block partials.

constexpr int kRedThreads = 256;
__global__ void __launch_bounds__(kRedThreads) reduce3_kernel(const double* a, const double* b, long n,
                                                              KSum* part) {
  __shared__ KSum sh[3][kRedThreads];
  KSum s0{0, 0}, s1{0, 0}, s2{0, 0};
  for (long i = blockIdx.x * long(kRedThreads) + threadIdx.x; i < n; i += long(gridDim.x) * kRedThreads) {
    double x = a[i];
    kadd(s0, x);
    kadd(s1, x * x);
    if (b) kadd(s2, b[i]);
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int k = 0; k < 3; ++k) kmerge(sh[k][threadIdx.x], sh[k][threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x < 3) part[blockIdx.x * 3 + threadIdx.x] = sh[threadIdx.x][0];
}
__global__ void __launch_bounds__(kRedThreads) reduce_parts_kernel(const KSum* part, int nb, double* out) {
  __shared__ KSum sh[3][kRedThreads];
  KSum s[3] = {{0, 0}, {0, 0}, {0, 0}};
  for (int b = threadIdx.x; b < nb; b += kRedThreads)
    for (int k = 0; k < 3; ++k) kmerge(s[k], part[b * 3 + k]);
  for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int k = 0; k < 3; ++k) kmerge(sh[k][threadIdx.x], sh[k][threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x < 3) out[threadIdx.x] = sh[threadIdx.x][0].s + sh[threadIdx.x][0].c;
}

// compute_flux_csda_direct (src/Geometry.jl:1126-1209): the two-layer CSDA
// flux in closed form (one range inversion per layer), thread per sample,
// with d/d rho in tangent mode.  Tables read from global memory (L1/L2).
__device__ __forceinline__ Dd range_g(const TabView& tv, int m, Dd E) {
  return interp_logE(tv, tv.col(m, DP_COL_E), tv.col(m, DP_COL_LOGE), tv.col(m, DP_COL_CSDA_R), E,
                     dlog(E), nullptr);
}
__device__ __forceinline__ Dd stop_g(const TabView& tv, int m, Dd E) {
  return interp_logE(tv, tv.col(m, DP_COL_E), tv.col(m, DP_COL_LOGE), tv.col(m, DP_COL_CSDA_S), E,
                     dlog(E), nullptr);
}
__device__ __forceinline__ Dd energy_g(const TabView& tv, int m, Dd X) {
  return inverse_range(tv.col(m, DP_COL_CSDA_R), tv.col(m, DP_COL_E), tv.col(m, DP_COL_LOGE), tv.n,
                       X, nullptr);
}
// compute_decay_weight_from_path (src/Geometry.jl:1083-1093)
__device__ __forceinline__ Dd decay_g(double mass, double ctau, Dd L, Dd Eavg) {
  Dd g = dd(1.0) + Eavg / mass;
  Dd b = dsqrt(dmax(dd(1.0) - dd(1.0) / (g * g), dd(1e-12)));
  return dexp(-L / (b * g * dd(ctau)));
}

struct DirectParams {
  TabView tab;
  int rock, air;
  double thickness, rho, elevation, H, mass, ctau;
  long n;
  const double *E, *q, *w;
  double *contrib, *dcontrib;
};

__global__ void __launch_bounds__(128) direct_kernel(DirectParams P) {
  const TabView& tv = P.tab;
  const double el = P.elevation * (kPi / 180.0);
  const double c = cos(kPi / 2 - el);  // cos(zenith) = sin(elevation)
  const double cs = fmax(fabs(c), 0.01);
  // compute_air_grammage (src/Geometry.jl:1043-1055)
  const double Xa =
      fmax((1.205 * 12e3 / cs) * (exp(-P.thickness / 12e3) - exp(-P.H / 12e3)), 0.0);
  const double cst = cos_theta_star(c), cs129 = pow(cst, 1.29);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < P.n; i += long(gridDim.x) * blockDim.x) {
    const Dd rho = dd(P.rho, 1.0);
    const Dd E0 = dd(P.E[i]);
    const Dd Xr = dd(P.thickness / cs) * rho;
    const Dd E1 = energy_g(tv, P.rock, range_g(tv, P.rock, E0) + Xr);
    double f = 0.0, df = 0.0;
    if (E1.v < 1e12 && isfinite(E1.v)) {
      const Dd wr = stop_g(tv, P.rock, E1) / stop_g(tv, P.rock, E0);
      const Dd dr = decay_g(P.mass, P.ctau, dd(P.thickness / cs), (E0 + E1) / 2.0);
      const Dd E2 = energy_g(tv, P.air, range_g(tv, P.air, E1) + dd(Xa));
      if (E2.v < 1e12 && isfinite(E2.v)) {
        const Dd wa = stop_g(tv, P.air, E2) / stop_g(tv, P.air, E1);
        const Dd da = decay_g(P.mass, P.ctau, dd((P.H - P.thickness) / cs), (E1 + E2) / 2.0);
        double dlogF;
        const double F = gccly_flux(cst, cs129, E2.v, P.q[i], &dlogF);
        const Dd wgt = wr * dr * wa * da;
        f = wgt.v * F;
        df = wgt.d * F + wgt.v * F * dlogF * E2.d;
      }
    }
    P.contrib[i] = P.w[i] * f;
    if (P.dcontrib) P.dcontrib[i] = P.w[i] * df;
  }
}

static int setup(dp_ctx* ctx, const dp_physics* ph, const dp_mc_params* p, CsdaParams& P) {
  if (!ctx || !ph || !p) return fail(ctx, DP_ERR_ARG, "null argument");
  int rock = p->rock_material, air = p->air_material;
  if (rock < 0) {
    rock = dp_physics_material_index(ph, "StandardRock");
    if (rock < 0) rock = 0;
  }
  if (air < 0) {
    air = dp_physics_material_index(ph, "Air");
    if (air < 0) air = ph->n_mat - 1;
  }
  if (rock >= ph->n_mat || air >= ph->n_mat) return fail(ctx, DP_ERR_ARG, "material index out of range");
  if (p->porous_material >= 0 && p->porous_thickness > 0.0 &&
      (p->porous_material >= ph->n_mat || !(p->porous_density > 0.0)))
    return fail(ctx, DP_ERR_ARG, "porous layer: material index out of range or density not positive");
  double tmax = ph->host[(size_t(0) * DP_NCOL + DP_COL_E) * ph->n + ph->n - 1];
  double thr = p->source_energy_max > 0.0 ? p->source_energy_max : std::fmin(1e9, tmax);
  if (!(thr > 0.0 && thr <= tmax))
    return fail(ctx, DP_ERR_ARG, "source_energy_max must be positive and within the physics energy grid");
  P = CsdaParams{};
  P.tab = ph->view;
  P.rock = rock;
  P.air = air;
  P.geo = csda_geo(p->rock_thickness, p->rock_density, p->elevation,
                   p->primary_altitude > 0.0 ? p->primary_altitude : 3e4);
  P.threshold = thr;
  P.low = p->energy_threshold_low > 0.0 ? p->energy_threshold_low : 100.0;
  P.mass = ph->settings.mass;
  P.ctau = ph->settings.ctau;
  P.err_flag = ctx->d_flag;
  P.step_cap = step_cap(ctx);
  P.wait_iters = stage_wait(ctx);
  return DP_OK;
}

// One wave of resident blocks whose threads stride over the histories (a
// grid of several partial waves idles SMs at its end).
static int launch(dp_ctx* ctx, CsdaParams& P, const dp_physics* ph32 = nullptr) {
  const int threads = ph32 ? 128 : kCsdaThreads;
  const size_t smem = ph32 ? size_t(2 * F_NCOL) * ph32->ld32 * sizeof(float)
                           : size_t(S_NCOL + D_NCOL) * P.tab.ld * sizeof(double);
  int per_sm = 0, n_sm = 0;
  if (ph32)
    DP_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, csda32_kernel, threads,
                                                                     smem));
  else
    DP_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, csda_mc_kernel,
                                                                     threads, smem));
  DP_CHECK_CUDA(ctx, cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
  long blocks = (P.n + threads - 1) / threads;
  blocks = std::min(blocks, long(std::max(per_sm, 1)) * n_sm);
  if (blocks < 1) blocks = 1;
  timed_begin(ctx);
  if (ph32)
    csda32_kernel<<<int(blocks), threads, smem, ctx->stream>>>(P, ph32->dev32, ph32->ld32);
  else
    csda_mc_kernel<<<int(blocks), threads, smem, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, ph32 ? "csda_mc32" : "csda_mc");
  return DP_OK;
}

static int check_flag(dp_ctx* ctx) {
  if (!ctx->blocking) return DP_OK;  // deferred to dp_sync
  int flag = 0;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
    return fail(ctx, DP_ERR_STATE, flag == 4 ? "a CSDA history reached the transport step cap"
                                             : "a table-staging wait exceeded its limit");
  }
  return DP_OK;
}

// CSDA histories of a batch of lines of sight (device records and running
// offsets): per-history w*flux and w*dflux/drho of the line's density.
int csda_los(dp_ctx* ctx, const dp_physics* ph, int rock, int air, double threshold, double low,
             uint64_t seed, const dp_los* los, const int64_t* off, long n_los, long n,
             double* contrib, double* dcontrib, int precision) {
  CsdaParams P{};
  P.tab = ph->view;
  P.rock = rock;
  P.air = air;
  P.threshold = threshold;
  P.low = low;
  P.mass = ph->settings.mass;
  P.ctau = ph->settings.ctau;
  P.err_flag = ctx->d_flag;
  P.step_cap = step_cap(ctx);
  P.wait_iters = stage_wait(ctx);
  P.seed = seed;
  P.n = n;
  P.los = los;
  P.los_off = off;
  P.n_los = n_los;
  P.contrib = contrib;
  P.dcontrib = dcontrib;
  return launch(ctx, P, precision == DP_PREC_MIXED ? ph : nullptr);
}

}  // namespace dp

using namespace dp;

extern "C" {

int dp_csda_flux_samples_dev(dp_ctx* ctx, const dp_physics* ph, const dp_mc_params* p, long n,
                             const double* E, const double* q, const double* w, double* contrib,
                             double* dcontrib, int32_t* steps) {
  CsdaParams P;
  int rc = setup(ctx, ph, p, P);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!E || !q || !w || !contrib))) return fail(ctx, DP_ERR_ARG, "bad sample arrays");
  if (n == 0) return DP_OK;
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  P.n = n;
  P.E = E;
  P.q = q;
  P.w = w;
  P.contrib = contrib;
  P.dcontrib = dcontrib;
  P.steps = steps;
  rc = launch(ctx, P, p->precision == DP_PREC_MIXED ? ph : nullptr);
  if (rc) return rc;
  return check_flag(ctx);
}

int dp_csda_flux_samples(dp_ctx* ctx, const dp_physics* ph, const dp_mc_params* p, long n,
                         const double* E, const double* q, const double* w, double* contrib,
                         double* dcontrib, int32_t* steps) {
  if (!ctx) return DP_ERR_ARG;
  if (n <= 0) return n == 0 ? DP_OK : fail(ctx, DP_ERR_ARG, "negative n");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  size_t nb = size_t(n) * sizeof(double);
  char* s = static_cast<char*>(scratch(ctx, 6 * nb + size_t(n) * 4));
  if (!s) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  double *dE = (double*)s, *dq = dE + n, *dw = dq + n, *dc = dw + n, *dd_ = dc + n;
  int32_t* ds = (int32_t*)(dd_ + n);
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dE, E, nb, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dq, q, nb, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dw, w, nb, cudaMemcpyHostToDevice, ctx->stream));
  int rc = dp_csda_flux_samples_dev(ctx, ph, p, n, dE, dq, dw, dc, dcontrib ? dd_ : nullptr,
                                    steps ? ds : nullptr);
  if (rc) return rc;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(contrib, dc, nb, cudaMemcpyDeviceToHost, ctx->stream));
  if (dcontrib) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dcontrib, dd_, nb, cudaMemcpyDeviceToHost, ctx->stream));
  if (steps) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(steps, ds, size_t(n) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return DP_OK;
}

int dp_csda_direct_samples(dp_ctx* ctx, const dp_physics* ph, const dp_mc_params* p, long n,
                           const double* E, const double* q, const double* w, double* contrib,
                           double* dcontrib) {
  CsdaParams S;
  int rc = setup(ctx, ph, p, S);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!E || !q || !w || !contrib))) return fail(ctx, DP_ERR_ARG, "bad sample arrays");
  if (n == 0) return DP_OK;
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  size_t nb = size_t(n) * sizeof(double);
  char* s = static_cast<char*>(scratch(ctx, 5 * nb));
  if (!s) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  double *dE = (double*)s, *dq = dE + n, *dw = dq + n, *dc = dw + n, *dd_ = dc + n;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dE, E, nb, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dq, q, nb, cudaMemcpyHostToDevice, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dw, w, nb, cudaMemcpyHostToDevice, ctx->stream));
  DirectParams P{};
  P.tab = ph->view;
  P.rock = S.rock;
  P.air = S.air;
  P.thickness = p->rock_thickness;
  P.rho = p->rock_density;
  P.elevation = p->elevation;
  P.H = p->primary_altitude > 0.0 ? p->primary_altitude : 3e4;
  P.mass = ph->settings.mass;
  P.ctau = ph->settings.ctau;
  P.n = n;
  P.E = dE;
  P.q = dq;
  P.w = dw;
  P.contrib = dc;
  P.dcontrib = dcontrib ? dd_ : nullptr;
  long blocks = std::min((n + 127) / 128, 152L * 16);
  timed_begin(ctx);
  direct_kernel<<<int(blocks), 128, 0, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  timed_end(ctx, "csda_direct");
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(contrib, dc, nb, cudaMemcpyDeviceToHost, ctx->stream));
  if (dcontrib) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(dcontrib, dd_, nb, cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return DP_OK;
}

int dp_mc_samples(dp_ctx* ctx, const dp_mc_params* p, long n, double* E, double* q, double* w) {
  if (!ctx || !p || n < 0 || !E || !q || !w) return fail(ctx, DP_ERR_ARG, "bad arguments");
  double emax = p->energy_max > p->energy_min ? p->energy_max : p->energy_min;
  for (long i = 0; i < n; ++i) mc_sample(p->seed, uint64_t(i), p->energy_min, emax, E + i, q + i, w + i);
  return DP_OK;
}

int dp_backward_mc(dp_ctx* ctx, const dp_physics* ph, const dp_mc_params* p, dp_mc_result* out) {
  CsdaParams P;
  int rc = setup(ctx, ph, p, P);
  if (rc) return rc;
  if (!out || p->n_samples <= 0) return fail(ctx, DP_ERR_ARG, "n_samples must be positive");
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  long n = p->n_samples;
  // stochastic transport first (its scratch is released before the CSDA pass);
  // a porous layer runs through the stochastic kernels (CSDA steps when
  // straggling and scattering are off), which model it
  const bool porous = p->porous_material >= 0 && p->porous_thickness > 0.0;
  if (porous && p->compute_gradient)
    return fail(ctx, DP_ERR_ARG, "the CSDA gradient has no porous layer");
  const bool stochastic = p->straggling || p->scattering || porous;
  dp_los_result st{};
  int st_rc = DP_OK;
  if (stochastic) {
    st_rc = mc_backward_stochastic(ctx, ph, p, P.rock, P.air, P.threshold, &st);
    if (st_rc && st_rc != DP_ERR_DOMAIN && st_rc != DP_ERR_STATE) return st_rc;
    if (!p->compute_gradient) {
      *out = dp_mc_result{};
      out->flux = st.flux;
      out->sigma = st.sigma;
      out->source_energy_max = P.threshold;
      out->n_samples = n;
      out->n_status_nonzero = st.n_status_nonzero;
      return st_rc;
    }
  }
  const int nb = 152 * 2;
  char* s = static_cast<char*>(scratch(ctx, size_t(n) * 2 * sizeof(double) + nb * 3 * sizeof(KSum) + 64));
  if (!s) return fail(ctx, DP_ERR_ALLOC, "scratch allocation failed");
  double* dc = (double*)s;
  double* dd_ = dc + n;
  KSum* part = (KSum*)(dd_ + n);
  double* sums = (double*)(part + nb * 3);
  P.n = n;
  P.use_philox = 1;
  P.seed = p->seed;
  P.emin = p->energy_min;
  P.emax = p->energy_max > p->energy_min ? p->energy_max : p->energy_min;
  P.contrib = dc;
  P.dcontrib = dd_;
  rc = launch(ctx, P, p->precision == DP_PREC_MIXED ? ph : nullptr);
  if (rc) return rc;
  reduce3_kernel<<<nb, kRedThreads, 0, ctx->stream>>>(dc, dd_, n, part);
  reduce_parts_kernel<<<1, kRedThreads, 0, ctx->stream>>>(part, nb, sums);
  ctx->launches += 2;
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  double h[3];
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  DP_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  rc = check_flag(ctx);
  if (rc) return rc;
  double flux = h[0] / n, var = h[1] / n - flux * flux;
  out->flux = flux;
  out->sigma = p->rock_thickness > 0.0 ? std::sqrt(std::fmax(var, 0.0) / n) : 0.0;
  out->gradient = p->compute_gradient ? h[2] / n : 0.0;
  out->gradient_flux = p->compute_gradient ? flux : 0.0;
  out->source_energy_max = P.threshold;
  out->n_samples = n;
  out->n_status_nonzero = 0;
  if (stochastic) {
    out->flux = st.flux;
    out->sigma = st.sigma;
    out->n_status_nonzero = st.n_status_nonzero;
    return st_rc;
  }
  return DP_OK;
}

}  // extern "C"

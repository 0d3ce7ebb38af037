// wtomo.cu -- the water-fraction CSDA forward model of src/Tomography.jl on
// the device: compute_directional_flux_csda (:667-727),
// directional_flux_and_grad_csda and assemble_forward_and_jacobian
// (:736-820), with the CSDA correction multipliers (:85-214, :367-412,
// :557-579).  FP64 (the reference's operations).
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

// ------------------------------------------------------------ N tangents
template <int N>
struct T {
  double v;
  double d[N];
};
template <int N> __device__ __forceinline__ T<N> cst(double v) {
  T<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N> __device__ __forceinline__ T<N> seed(double v, int i) {
  T<N> r = cst<N>(v);
  r.d[i] = 1.0;
  return r;
}
template <int N> __device__ __forceinline__ T<N> operator+(T<N> a, T<N> b) {
  T<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ T<N> operator-(T<N> a, T<N> b) {
  T<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ T<N> operator-(T<N> a) {
  T<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ T<N> operator*(T<N> a, T<N> b) {
  T<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ T<N> operator*(double a, T<N> b) {
  T<N> r;
  r.v = a * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a * b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ T<N> operator/(T<N> a, T<N> b) {
  T<N> r;
  r.v = a.v / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
  return r;
}
template <int N> __device__ __forceinline__ T<N> texp(T<N> a) {
  T<N> r;
  r.v = exp(a.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = r.v * a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ T<N> tlog(T<N> a) {
  T<N> r;
  r.v = log(a.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / a.v;
  return r;
}
template <int N> __device__ __forceinline__ T<N> tsqrt(T<N> a) {
  T<N> r;
  r.v = sqrt(a.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / (2.0 * r.v);
  return r;
}
// Julia min/max: the left operand on ties, compared by value (_csda_min/_csda_max)
template <int N> __device__ __forceinline__ T<N> tmin(T<N> a, T<N> b) { return b.v < a.v ? b : a; }
template <int N> __device__ __forceinline__ T<N> tmax(T<N> a, T<N> b) { return b.v > a.v ? b : a; }

// ------------------------------------------------------------ run constants
struct Params {
  TabView tv;              // FP64 tables in global memory (grid layout)
  const double* col[12];   // the staged columns (global addresses)
  uint32_t col_bytes;
  int porous;              // porous material present
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
};
// Staged column slots: energies, log energies, then per material
// (rock, water, porous) CSDA and restricted stopping power and straggling,
// then the air's CSDA stopping power.
enum Slot { S_E = 0, S_LE, R_CS, R_MS, R_ST, W_CS, W_MS, W_ST, P_CS, P_MS, P_ST, A_CS, kSlots };

struct Tables {
  const double* c[kSlots];
  int n, uniform;
  double lE0, inv_dlE;
};

// Interval and offset of E on the grid (src/Physics.jl:660-687); the value
// and its tangents are linear in log E.
template <int N>
struct At {
  int i;        // -1 below, -2 above the grid
  T<N> t;       // (log E - log E_i) / (log E_(i+1) - log E_i)
};
template <int N>
__device__ __forceinline__ At<N> locate(const Tables& tb, T<N> E) {
  At<N> a;
  const int n = tb.n;
  if (E.v <= tb.c[S_E][0]) {
    a.i = -1;
    return a;
  }
  if (E.v >= tb.c[S_E][n - 1]) {
    a.i = -2;
    return a;
  }
  T<N> lE = tlog(E);
  const double* lx = tb.c[S_LE];
  a.i = tb.uniform ? uniform_interval(lx, n, lE.v, tb.lE0, tb.inv_dlE) : bisect(lx, n, lE.v);
  a.t = (lE - cst<N>(lx[a.i])) / cst<N>(lx[a.i + 1] - lx[a.i]);
  return a;
}
template <int N>
__device__ __forceinline__ T<N> at(const Tables& tb, const At<N>& a, int slot) {
  const double* y = tb.c[slot];
  if (a.i == -1) return cst<N>(y[0]);
  if (a.i == -2) return cst<N>(y[tb.n - 1]);
  return cst<N>(y[a.i]) + a.t * cst<N>(y[a.i + 1] - y[a.i]);
}

// A cell's material: water fraction w, porous top layer or not.
template <int N>
struct Cell {
  T<N> w;
  bool porous;
};
// cell_density / cell_stopping_power / cell_straggling / cell_hardloss
// (src/Tomography.jl:303-352)
template <int N>
__device__ __forceinline__ T<N> cell_density(const Params& P, const Cell<N>& c) {
  const T<N> one = cst<N>(1.0);
  if (c.porous)
    return one / (0.5 * (one - c.w) / cst<N>(P.rho_porous) +
                  0.5 * (one - c.w) / cst<N>(P.rho_rock) + c.w / cst<N>(P.rho_water));
  return one / ((one - c.w) / cst<N>(P.rho_rock) + c.w / cst<N>(P.rho_water));
}
template <int N>
__device__ __forceinline__ T<N> cell_mix(const Cell<N>& c, T<N> r, T<N> w, T<N> p) {
  const T<N> one = cst<N>(1.0);
  if (c.porous) return 0.5 * (one - c.w) * p + 0.5 * (one - c.w) * r + c.w * w;
  return (one - c.w) * r + c.w * w;
}
template <int N>
__device__ __forceinline__ T<N> cell_S(const Tables& tb, const Cell<N>& c, T<N> E) {
  At<N> a = locate(tb, E);
  return cell_mix(c, at(tb, a, R_CS), at(tb, a, W_CS), c.porous ? at(tb, a, P_CS) : cst<N>(0.0));
}

// compute_decay_weight_from_path (src/Geometry.jl:1083-1107)
template <int N>
__device__ __forceinline__ T<N> decay(const Params& P, T<N> L, T<N> Eavg) {
  const T<N> one = cst<N>(1.0);
  T<N> g = one + Eavg / cst<N>(P.mass);
  T<N> b2 = one - one / (g * g);
  T<N> b = tsqrt(b2.v >= 1e-12 ? b2 : cst<N>(1e-12));
  return texp(-L / (b * g * cst<N>(P.ctau)));
}

// One Heun step (src/Tomography.jl:455-471); false on an invalid step.
template <int N, class SF>
__device__ __forceinline__ bool heun(const Params& P, SF S, T<N> dedx0, T<N> ds, T<N> density,
                                     T<N>& E, T<N>& W) {
  T<N> gx = ds * density;
  T<N> Ep = E + dedx0 * gx;
  T<N> dedx1 = S(Ep);
  T<N> En = E + 0.5 * (dedx0 + dedx1) * gx;
  if (!isfinite(En.v) || En.v >= 1e12) return false;
  T<N> dedxn = S(En);
  W = W * (dedxn / tmax(dedx0, cst<N>(1e-30)));
  W = W * decay(P, ds, 0.5 * (E + En));
  E = En;
  return true;
}

// propagate_csda_cell_segment / propagate_csda_uniform_segment (:444-509)
template <int N, class SF>
__device__ bool solid_segment(const Params& P, SF S, T<N> density, double distance, T<N>& E,
                              T<N>& W) {
  T<N> remaining = cst<N>(distance);
  for (int guard = 0; remaining.v > 1e-8; ++guard) {
    if (guard > 10000000) return false;
    T<N> dedx0 = S(E);
    if (!isfinite(dedx0.v) || dedx0.v <= 0.0) return false;
    T<N> grel = kMaxGain * tmax(E, cst<N>(1e-6)) / dedx0;
    T<N> gstep = tmin(tmin(remaining * density, tmax(grel, cst<N>(1e-6))), kMaxStep * density);
    T<N> ds = tmin(remaining, gstep / tmax(density, cst<N>(1e-12)));
    if (ds.v <= 0.0) return false;
    if (!heun(P, S, dedx0, ds, density, E, W)) return false;
    remaining = remaining - ds;
  }
  return true;
}

// propagate_csda_air_segment (:516-551): remaining and traversed carry the
// steps' tangents, and with them the altitude of the density.
template <int N>
__device__ bool air_segment(const Params& P, const Tables& tb, double start_z, double cos_t,
                            double distance, T<N>& E, T<N>& W) {
  auto S = [&](T<N> e) { return at(tb, locate(tb, e), A_CS); };
  T<N> remaining = cst<N>(distance), traversed = cst<N>(0.0);
  const T<N> base = cst<N>(P.det_elev + start_z), ct = cst<N>(cos_t);
  for (int guard = 0; remaining.v > 1e-8; ++guard) {
    if (guard > 10000000) return false;
    T<N> alt = base + ct * (traversed + 0.5 * tmin(remaining, cst<N>(kMaxStep)));
    T<N> rho = 1.205 * texp(-alt / cst<N>(12e3));
    T<N> dedx0 = S(E);
    if (!isfinite(dedx0.v) || dedx0.v <= 0.0) return false;
    T<N> grel = kMaxGain * tmax(E, cst<N>(1e-6)) / dedx0;
    T<N> ds = tmin(tmin(remaining, cst<N>(kMaxStep)), grel / tmax(rho, cst<N>(1e-12)));
    ds = tmax(ds, cst<N>(1e-3));
    alt = base + ct * (traversed + 0.5 * ds);
    rho = 1.205 * texp(-alt / cst<N>(12e3));
    if (!heun(P, S, dedx0, ds, rho, E, W)) return false;
    traversed = traversed + ds;
    remaining = remaining - ds;
  }
  return true;
}

// Straggling and hard-loss increments of a segment at its mean energy
// (src/Tomography.jl:598-617): V += Omega(e_rep) gx, H += (S_csda - S_mixed) gx.
template <int N>
__device__ __forceinline__ void vh_cell(const Tables& tb, const Cell<N>& c, T<N> e_rep, T<N> gx,
                                        T<N>& v, T<N>& h) {
  At<N> a = locate(tb, e_rep);
  const T<N> z = cst<N>(0.0);
  v = cell_mix(c, at(tb, a, R_ST), at(tb, a, W_ST), c.porous ? at(tb, a, P_ST) : z) * gx;
  h = cell_mix(c, at(tb, a, R_CS) - at(tb, a, R_MS), at(tb, a, W_CS) - at(tb, a, W_MS),
               c.porous ? at(tb, a, P_CS) - at(tb, a, P_MS) : z) * gx;
}
template <int N>
__device__ __forceinline__ void vh_rock(const Tables& tb, T<N> e_rep, T<N> gx, T<N>& v, T<N>& h) {
  At<N> a = locate(tb, e_rep);
  v = at(tb, a, R_ST) * gx;
  h = (at(tb, a, R_CS) - at(tb, a, R_MS)) * gx;
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

// Per-sample results of pass 1.
struct Lane {
  double f;       // w * corr * flux_gccly of the sample (0 when the walk is invalid)
  double A;       // lambda_N P_N + C_N (+ alpha terms)
  double aV, aH;  // d log corr / dV, d log corr / dH
};

__device__ __forceinline__ bool cell_porous(const Params& P, int cell) {
  return P.porous && P.porous_top > 0.0 && P.shallow && P.shallow[cell];
}

// Pass 1: flux of one sample and its end-of-path adjoint constants.
__device__ Lane pass1(const Params& P, const Tables& tb, long b, double E0, double q) {
  Lane out{0.0, 0.0, 0.0, 0.0};
  const double ct = P.cos_t[b];
  double E = E0, W = 1.0, V = 0.0, H = 0.0;
  double Pk = 1.0, Cs = 0.0, Cv = 0.0, Ch = 0.0;
  const int64_t s0 = P.seg_ptr[b], s1 = P.seg_ptr[b + 1];
  for (int64_t k = s0; k < s1; ++k) {
    const int cell = P.seg_cell[k];
    Cell<1> c{cst<1>(P.wf[cell]), cell_porous(P, cell)};
    T<1> rho = cell_density(P, c);
    T<1> e = seed<1>(E, 0), g = cst<1>(1.0);
    const T<1> e_in = e;
    if (!solid_segment(P, [&](T<1> x) { return cell_S(tb, c, x); }, rho, P.seg_len[k], e, g))
      return out;
    T<1> v, h;
    vh_cell(tb, c, 0.5 * (e_in + e), P.seg_len[k] * rho, v, h);
    Cs += (g.d[0] / g.v) * Pk;
    Cv += v.d[0] * Pk;
    Ch += h.d[0] * Pk;
    Pk *= e.d[0];
    E = e.v;
    W *= g.v;
    V += v.v;
    H += h.v;
  }
  if (P.rem[b] > 1e-8) {
    T<1> e = seed<1>(E, 0), g = cst<1>(1.0);
    const T<1> e_in = e;
    auto S = [&](T<1> x) { return at(tb, locate(tb, x), R_CS); };
    if (!solid_segment(P, S, cst<1>(P.rho_rock), P.rem[b], e, g)) return out;
    T<1> v, h;
    vh_rock(tb, 0.5 * (e_in + e), cst<1>(P.rem[b] * P.rho_rock), v, h);
    Cs += (g.d[0] / g.v) * Pk;
    Cv += v.d[0] * Pk;
    Ch += h.d[0] * Pk;
    Pk *= e.d[0];
    E = e.v;
    W *= g.v;
    V += v.v;
    H += h.v;
  }
  {
    T<1> e = seed<1>(E, 0), g = cst<1>(1.0);
    const double air = fmax(0.0, P.primary - P.exit_z[b]) / fmax(ct, 1e-3);
    if (!air_segment(P, tb, P.exit_z[b], ct, air, e, g)) return out;
    Cs += (g.d[0] / g.v) * Pk;
    Pk *= e.d[0];
    E = e.v;
    W *= g.v;
  }
  const double cs = cos_theta_star(ct), cs129 = pow(cs, 1.29);
  double dlogF;
  const double F = gccly_flux(cs, cs129, E, q, &dlogF);
  double corr = 1.0, dcorr = 0.0;
  if (P.corr) {
    // csda_var_correction (:384-391)
    const double e = fmax(E, 1.0);
    double bi, dbi;
    spectral_index(e, cs, cs129, &bi, &dbi);
    const double cstr = 0.5 * bi * (bi + 1.0), Hp = fmax(H, 0.0);
    corr = exp(P.ks * cstr * V / (e * e) - P.kh * Hp / e);
    out.aV = P.ks * cstr / (e * e);
    out.aH = H > 0.0 ? -P.kh / e : 0.0;
    if (E > 1.0)
      dcorr = P.ks * V * ((bi + 0.5) * dbi / (e * e) - 2.0 * cstr / (e * e * e)) + P.kh * Hp / (e * e);
  }
  out.f = W * corr * F;
  out.A = (dlogF + dcorr) * Pk + Cs + out.aV * Cv + out.aH * Ch;
  return out;
}

// Deterministic warp sum (fixed shuffle tree).
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__global__ void __launch_bounds__(kThreads) wtomo_kernel(const __grid_constant__ Params P) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  double* cols = reinterpret_cast<double*>(smem + 16);
  if (!stage_columns(cols, P.col, kSlots, P.col_bytes, bar)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    return;
  }
  Tables tb;
  const int ld = int(P.col_bytes / 8);
#pragma unroll
  for (int s = 0; s < kSlots; ++s) tb.c[s] = cols + size_t(s) * ld;
  tb.n = P.tv.n;
  tb.uniform = P.tv.uniform;
  tb.lE0 = P.tv.lE0;
  tb.inv_dlE = P.tv.inv_dlE;

  const int lane = threadIdx.x & 31;
  const long warps = long(gridDim.x) * (kThreads / 32);
  const int n_chunks = (P.n_e + 31) / 32;
  for (long b = long(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5); b < P.n_bins; b += warps) {
    const int64_t s0 = P.seg_ptr[b], s1 = P.seg_ptr[b + 1];
    const double ct = P.cos_t[b];
    // device-array calls: cells outside the water-fraction vector end the call
    bool bad = false;
    for (int64_t k = s0 + lane; k < s1; k += 32) bad |= P.seg_cell[k] < 0 || P.seg_cell[k] >= P.n_cells;
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) {
        P.flux[b] = CUDART_NAN;
        atomicExch(P.err_flag, 3);
      }
      continue;
    }
    if ((P.valid && !P.valid[b]) || !(ct > 0.0)) {
      if (lane == 0) P.flux[b] = CUDART_NAN;
      if (P.jac)
        for (int64_t k = s0 + lane; k < s1; k += 32) P.jac[k] = 0.0;
      continue;
    }
    // pass 1 over the samples
    Lane L[kMaxChunks];
    double sum = 0.0;
#pragma unroll
    for (int ch = 0; ch < kMaxChunks; ++ch) {
      L[ch] = Lane{0.0, 0.0, 0.0, 0.0};
      const int s = ch * 32 + lane;
      if (ch < n_chunks && s < P.n_e) {
        L[ch] = pass1(P, tb, b, P.E[s], P.q[s]);
        L[ch].f *= 2.0 * P.ew[s];
      }
      sum += L[ch].f;
    }
    sum = warp_sum(sum);
    // geometric and material multipliers (:405-412, :557-579)
    double Lsum = 0.0, water = 0.0, mass = 0.0;
    for (int64_t k = s0 + lane; k < s1; k += 32) {
      const int cell = P.seg_cell[k];
      Cell<1> c{cst<1>(P.wf[cell]), cell_porous(P, cell)};
      const double gx = P.seg_len[k] * cell_density(P, c).v;
      Lsum += P.seg_len[k];
      water += P.wf[cell] * gx;
      mass += gx;
    }
    Lsum = warp_sum(Lsum);
    water = warp_sum(water);
    mass = warp_sum(mass) + P.rem[b] * P.rho_rock;
    double G = 1.0;
    if (P.corr && (P.ra != 0.0 || P.rb != 0.0 || P.rc != 0.0 || P.rd != 0.0)) {
      const double lL = log(fmax(P.rem[b] + Lsum, 1.0));
      G = exp(P.ra + P.rb * lL + P.rc * lL * lL + P.rd * ct);
    }
    const double qf = water / fmax(mass, 1e-30);
    const double M = P.mcorr ? exp(P.lin * qf + P.quad * qf * qf) : 1.0;
    const double flux = G * M * sum / double(P.n_e);
    if (lane == 0) P.flux[b] = flux;
    if (!P.jac) continue;

    // pass 2: d log f / d w per cell segment, summed over the samples
    const double scale = G * M / double(P.n_e);
    for (int ch = 0; ch < n_chunks; ++ch) {
      const int s = ch * 32 + lane;
      const Lane& l = L[ch];
      const bool active = s < P.n_e && l.f != 0.0;
      double E = active ? P.E[s] : 0.0;
      double Pk = 1.0, Cs = 0.0, Cv = 0.0, Ch = 0.0;
      bool alive = active;
      for (int64_t k = s0; k < s1; ++k) {
        double gk = 0.0;
        if (alive) {
          const int cell = P.seg_cell[k];
          Cell<2> c{seed<2>(P.wf[cell], 1), cell_porous(P, cell)};
          T<2> rho = cell_density(P, c);
          T<2> e = seed<2>(E, 0), g = cst<2>(1.0);
          const T<2> e_in = e;
          if (solid_segment(P, [&](T<2> x) { return cell_S(tb, c, x); }, rho, P.seg_len[k], e, g)) {
            T<2> v, h;
            vh_cell(tb, c, 0.5 * (e_in + e), P.seg_len[k] * rho, v, h);
            Cs += (g.d[0] / g.v) * Pk;
            Cv += v.d[0] * Pk;
            Ch += h.d[0] * Pk;
            Pk *= e.d[0];
            const double lam = (l.A - Cs - l.aV * Cv - l.aH * Ch) / Pk;
            gk = l.f * (lam * e.d[1] + g.d[1] / g.v + l.aV * v.d[1] + l.aH * h.d[1]);
            E = e.v;
          } else {
            alive = false;  // not reached: pass 1 saw the same valid walk
          }
        }
        gk = warp_sum(gk);
        if (lane == 0) P.jac[k] = (ch ? P.jac[k] : 0.0) + scale * gk;
      }
    }
    // d M / d w through the column water fraction q (:557-579)
    if (P.mcorr) {
      const double dlogM = P.lin + 2.0 * P.quad * qf, mm = fmax(mass, 1e-30);
      __syncwarp();
      for (int64_t k = s0 + lane; k < s1; k += 32) {
        const int cell = P.seg_cell[k];
        Cell<2> c{seed<2>(P.wf[cell], 1), cell_porous(P, cell)};
        const T<2> rho = cell_density(P, c);
        const double gx = P.seg_len[k] * rho.v, dgx = P.seg_len[k] * rho.d[1];
        const double dwater = gx + P.wf[cell] * dgx;
        const double dq = mass > 1e-30 ? (dwater * mm - water * dgx) / (mm * mm) : dwater / mm;
        P.jac[k] += flux * dlogM * dq;
      }
    }
  }
}

}  // namespace wt
}  // namespace dp

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
        long n_cells, const uint8_t* shallow, const double* wf, double* flux, double* jac) {
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
  const size_t smem = 16 + size_t(wt::kSlots) * P.col_bytes;
  DP_CHECK_CUDA(ctx, cudaFuncSetAttribute(wt::wtomo_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          int(smem)));
  int per_sm = 0, n_sm = 0;
  DP_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wt::wtomo_kernel,
                                                                   wt::kThreads, smem));
  DP_CHECK_CUDA(ctx, cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
  const long need = (B->n_bins + wt::kThreads / 32 - 1) / (wt::kThreads / 32);
  const long blocks = std::max(1L, std::min(need, long(std::max(per_sm, 1)) * n_sm));
  timed_begin(ctx);
  wt::wtomo_kernel<<<int(blocks), wt::kThreads, smem, ctx->stream>>>(P);
  DP_CHECK_CUDA(ctx, cudaGetLastError());
  ++ctx->launches;
  timed_end(ctx, jac ? "dir_csda_grad" : "dir_csda");
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
                    const double* water_fraction, double* flux, double* jac) {
  if (!ctx || !ph || !batch || !water_fraction || !flux || batch->n_bins < 0 || n_cells < 0)
    return fail(ctx, DP_ERR_ARG, "bad arguments");
  if (batch->n_bins == 0) return DP_OK;
  DP_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  int rc = run(ctx, ph, cfg, batch, n_cells, shallow, water_fraction, flux, jac);
  if (rc) return rc;
  return ctx->blocking ? read_flag(ctx) : DP_OK;
}

int dp_dir_csda(dp_ctx* ctx, const dp_physics* ph, const dp_csda_config* cfg,
                const dp_csda_batch* B, long n_cells, const uint8_t* shallow,
                const double* water_fraction, double* flux, double* jac) {
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
  int rc = run(ctx, ph, cfg, &D, n_cells, sh, w, fl, jc);
  if (rc) return rc;
  DP_CHECK_CUDA(ctx, cudaMemcpyAsync(flux, fl, db, cudaMemcpyDeviceToHost, s));
  if (jac && ns) DP_CHECK_CUDA(ctx, cudaMemcpyAsync(jac, jc, size_t(ns) * 8, cudaMemcpyDeviceToHost, s));
  return read_flag(ctx);
}

}  // extern "C"

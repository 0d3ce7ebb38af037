// wtomo_walk.cuh -- the CSDA walk and the kernel of wtomo.cu in one scalar
// type.  wtomo.cu includes it twice: WT_REAL double (the reference's FP64
// operations) and WT_REAL float (FP32 steps and tangents; the prefix sums of
// the adjoint, the flux and the reductions stay FP64).  No include guard on
// purpose; WT_NS names the namespace of each instance.

namespace dp {
namespace WT_NS {

using Real = WT_REAL;
using wt::Lane;
using wt::Params;
using wt::kMaxChunks;
using wt::kThreads;

// ------------------------------------------------------------ N tangents
template <int N>
struct T {
  Real v;
  Real d[N];
};
template <int N> __device__ __forceinline__ T<N> cst(Real v) {
  T<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = Real(0);
  return r;
}
template <int N> __device__ __forceinline__ T<N> seed(Real v, int i) {
  T<N> r = cst<N>(v);
  r.d[i] = Real(1);
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
template <int N> __device__ __forceinline__ T<N> operator*(Real a, T<N> b) {
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
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / (Real(2) * r.v);
  return r;
}
// Julia min/max: the left operand on ties, compared by value (_csda_min/_csda_max)
template <int N> __device__ __forceinline__ T<N> tmin(T<N> a, T<N> b) { return b.v < a.v ? b : a; }
template <int N> __device__ __forceinline__ T<N> tmax(T<N> a, T<N> b) { return b.v > a.v ? b : a; }

// Run constants in the walk's precision (converted once per thread).
struct Consts {
  Real mass, ctau, rho_rock, rho_water, rho_porous, det_elev;
};

struct Tables {
  const Real* c[wt::kSlots];
  int n, uniform;
  Real lE0, inv_dlE;
};

// Interval and offset of E on the grid (src/Physics.jl:660-687); the value
// and its tangents are linear in log E.
template <int N>
struct At {
  int i;   // -1 below, -2 above the grid
  T<N> t;  // (log E - log E_i) / (log E_(i+1) - log E_i)
};
template <int N>
__device__ __forceinline__ At<N> locate(const Tables& tb, T<N> E) {
  At<N> a;
  const int n = tb.n;
  if (E.v <= tb.c[wt::S_E][0]) {
    a.i = -1;
    return a;
  }
  if (E.v >= tb.c[wt::S_E][n - 1]) {
    a.i = -2;
    return a;
  }
  T<N> lE = tlog(E);
  const Real* lx = tb.c[wt::S_LE];
  int i;
  if (tb.uniform) {
    // O(1) guess, corrected to the bisection answer
    Real f = floor((lE.v - tb.lE0) * tb.inv_dlE);
    i = f < Real(0) ? 0 : (f > Real(n - 2) ? n - 2 : int(f));
    while (i > 0 && lE.v < lx[i]) --i;
    while (i < n - 2 && !(lE.v < lx[i + 1])) ++i;
  } else {
    int lo = 0, hi = n - 1;
    while (lo < hi - 1) {
      int mid = (lo + hi) >> 1;
      if (lE.v < lx[mid]) hi = mid; else lo = mid;
    }
    i = lo;
  }
  a.i = i;
  a.t = (lE - cst<N>(lx[i])) / cst<N>(lx[i + 1] - lx[i]);
  return a;
}
template <int N>
__device__ __forceinline__ T<N> at(const Tables& tb, const At<N>& a, int slot) {
  const Real* y = tb.c[slot];
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
__device__ __forceinline__ T<N> cell_density(const Consts& k, const Cell<N>& c) {
  const T<N> one = cst<N>(Real(1));
  if (c.porous)
    return one / (Real(0.5) * (one - c.w) / cst<N>(k.rho_porous) +
                  Real(0.5) * (one - c.w) / cst<N>(k.rho_rock) + c.w / cst<N>(k.rho_water));
  return one / ((one - c.w) / cst<N>(k.rho_rock) + c.w / cst<N>(k.rho_water));
}
template <int N>
__device__ __forceinline__ T<N> cell_mix(const Cell<N>& c, T<N> r, T<N> w, T<N> p) {
  const T<N> one = cst<N>(Real(1));
  if (c.porous) return Real(0.5) * (one - c.w) * p + Real(0.5) * (one - c.w) * r + c.w * w;
  return (one - c.w) * r + c.w * w;
}
template <int N>
__device__ __forceinline__ T<N> cell_S(const Tables& tb, const Cell<N>& c, T<N> E) {
  At<N> a = locate(tb, E);
  return cell_mix(c, at(tb, a, wt::R_CS), at(tb, a, wt::W_CS),
                  c.porous ? at(tb, a, wt::P_CS) : cst<N>(Real(0)));
}

// compute_decay_weight_from_path (src/Geometry.jl:1083-1107)
template <int N>
__device__ __forceinline__ T<N> decay(const Consts& k, T<N> L, T<N> Eavg) {
  const T<N> one = cst<N>(Real(1));
  T<N> g = one + Eavg / cst<N>(k.mass);
  T<N> b2 = one - one / (g * g);
  T<N> b = tsqrt(b2.v >= Real(1e-12) ? b2 : cst<N>(Real(1e-12)));
  return texp(-L / (b * g * cst<N>(k.ctau)));
}

// One Heun step (src/Tomography.jl:455-471); false on an invalid step.
template <int N, class SF>
__device__ __forceinline__ bool heun(const Consts& k, SF S, T<N> dedx0, T<N> ds, T<N> density,
                                     T<N>& E, T<N>& W) {
  T<N> gx = ds * density;
  T<N> Ep = E + dedx0 * gx;
  T<N> dedx1 = S(Ep);
  T<N> En = E + Real(0.5) * (dedx0 + dedx1) * gx;
  if (!isfinite(En.v) || En.v >= Real(1e12)) return false;
  T<N> dedxn = S(En);
  W = W * (dedxn / tmax(dedx0, cst<N>(Real(1e-30))));
  W = W * decay(k, ds, Real(0.5) * (E + En));
  E = En;
  return true;
}

// propagate_csda_cell_segment / propagate_csda_uniform_segment (:444-509)
template <int N, class SF>
__device__ bool solid_segment(const Consts& k, SF S, T<N> density, Real distance, T<N>& E,
                              T<N>& W) {
  T<N> remaining = cst<N>(distance);
  for (int guard = 0; remaining.v > Real(1e-8); ++guard) {
    if (guard > 10000000) return false;
    T<N> dedx0 = S(E);
    if (!isfinite(dedx0.v) || dedx0.v <= Real(0)) return false;
    T<N> grel = Real(wt::kMaxGain) * tmax(E, cst<N>(Real(1e-6))) / dedx0;
    T<N> gstep = tmin(tmin(remaining * density, tmax(grel, cst<N>(Real(1e-6)))),
                      Real(wt::kMaxStep) * density);
    T<N> ds = tmin(remaining, gstep / tmax(density, cst<N>(Real(1e-12))));
    if (ds.v <= Real(0)) return false;
    if (!heun(k, S, dedx0, ds, density, E, W)) return false;
    remaining = remaining - ds;
  }
  return true;
}

// propagate_csda_air_segment (:516-551): remaining and traversed carry the
// steps' tangents, and with them the altitude of the density.
template <int N>
__device__ bool air_segment(const Consts& k, const Tables& tb, Real start_z, Real cos_t,
                            Real distance, T<N>& E, T<N>& W) {
  auto S = [&](T<N> e) { return at(tb, locate(tb, e), wt::A_CS); };
  T<N> remaining = cst<N>(distance), traversed = cst<N>(Real(0));
  const T<N> base = cst<N>(k.det_elev + start_z), ct = cst<N>(cos_t);
  const T<N> H = cst<N>(Real(12e3));
  for (int guard = 0; remaining.v > Real(1e-8); ++guard) {
    if (guard > 10000000) return false;
    T<N> alt = base + ct * (traversed + Real(0.5) * tmin(remaining, cst<N>(Real(wt::kMaxStep))));
    T<N> rho = Real(1.205) * texp(-alt / H);
    T<N> dedx0 = S(E);
    if (!isfinite(dedx0.v) || dedx0.v <= Real(0)) return false;
    T<N> grel = Real(wt::kMaxGain) * tmax(E, cst<N>(Real(1e-6))) / dedx0;
    T<N> ds = tmin(tmin(remaining, cst<N>(Real(wt::kMaxStep))),
                   grel / tmax(rho, cst<N>(Real(1e-12))));
    ds = tmax(ds, cst<N>(Real(1e-3)));
    alt = base + ct * (traversed + Real(0.5) * ds);
    rho = Real(1.205) * texp(-alt / H);
    if (!heun(k, S, dedx0, ds, rho, E, W)) return false;
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
  const T<N> z = cst<N>(Real(0));
  v = cell_mix(c, at(tb, a, wt::R_ST), at(tb, a, wt::W_ST), c.porous ? at(tb, a, wt::P_ST) : z) *
      gx;
  h = cell_mix(c, at(tb, a, wt::R_CS) - at(tb, a, wt::R_MS),
               at(tb, a, wt::W_CS) - at(tb, a, wt::W_MS),
               c.porous ? at(tb, a, wt::P_CS) - at(tb, a, wt::P_MS) : z) *
      gx;
}
template <int N>
__device__ __forceinline__ void vh_rock(const Tables& tb, T<N> e_rep, T<N> gx, T<N>& v, T<N>& h) {
  At<N> a = locate(tb, e_rep);
  v = at(tb, a, wt::R_ST) * gx;
  h = (at(tb, a, wt::R_CS) - at(tb, a, wt::R_MS)) * gx;
}

// Pass 1: flux of one sample and its end-of-path adjoint constants.  The
// per-segment partials are accumulated in FP64.
__device__ Lane pass1(const Params& P, const Consts& k, const Tables& tb, long b, double E0,
                      double q) {
  Lane out{0.0, 0.0, 0.0, 0.0};
  const double ct = P.cos_t[b];
  Real E = Real(E0), W = Real(1), V = Real(0), H = Real(0);
  double Pk = 1.0, Cs = 0.0, Cv = 0.0, Ch = 0.0;
  const int64_t s0 = P.seg_ptr[b], s1 = P.seg_ptr[b + 1];
  for (int64_t j = s0; j < s1; ++j) {
    const int cell = P.seg_cell[j];
    Cell<1> c{cst<1>(Real(P.wf[cell])), wt::cell_porous(P, cell)};
    T<1> rho = cell_density(k, c);
    T<1> e = seed<1>(E, 0), g = cst<1>(Real(1));
    const T<1> e_in = e;
    const Real len = Real(P.seg_len[j]);
    if (!solid_segment(k, [&](T<1> x) { return cell_S(tb, c, x); }, rho, len, e, g)) return out;
    T<1> v, h;
    vh_cell(tb, c, Real(0.5) * (e_in + e), len * rho, v, h);
    Cs += double(g.d[0] / g.v) * Pk;
    Cv += double(v.d[0]) * Pk;
    Ch += double(h.d[0]) * Pk;
    Pk *= double(e.d[0]);
    E = e.v;
    W *= g.v;
    V += v.v;
    H += h.v;
  }
  if (P.rem[b] > 1e-8) {
    T<1> e = seed<1>(E, 0), g = cst<1>(Real(1));
    const T<1> e_in = e;
    auto S = [&](T<1> x) { return at(tb, locate(tb, x), wt::R_CS); };
    if (!solid_segment(k, S, cst<1>(k.rho_rock), Real(P.rem[b]), e, g)) return out;
    T<1> v, h;
    vh_rock(tb, Real(0.5) * (e_in + e), cst<1>(Real(P.rem[b]) * k.rho_rock), v, h);
    Cs += double(g.d[0] / g.v) * Pk;
    Cv += double(v.d[0]) * Pk;
    Ch += double(h.d[0]) * Pk;
    Pk *= double(e.d[0]);
    E = e.v;
    W *= g.v;
    V += v.v;
    H += h.v;
  }
  {
    T<1> e = seed<1>(E, 0), g = cst<1>(Real(1));
    const double air = fmax(0.0, P.primary - P.exit_z[b]) / fmax(ct, 1e-3);
    if (!air_segment(k, tb, Real(P.exit_z[b]), Real(ct), Real(air), e, g)) return out;
    Cs += double(g.d[0] / g.v) * Pk;
    Pk *= double(e.d[0]);
    E = e.v;
    W *= g.v;
  }
  const double cs = cos_theta_star(ct), cs129 = pow(cs, 1.29);
  double dlogF;
  const double Ed = double(E), Vd = double(V), Hd = double(H);
  const double F = gccly_flux(cs, cs129, Ed, q, &dlogF);
  double corr = 1.0, dcorr = 0.0;
  if (P.corr) {
    // csda_var_correction (:384-391)
    const double e = fmax(Ed, 1.0);
    double bi, dbi;
    wt::spectral_index(e, cs, cs129, &bi, &dbi);
    const double cstr = 0.5 * bi * (bi + 1.0), Hp = fmax(Hd, 0.0);
    corr = exp(P.ks * cstr * Vd / (e * e) - P.kh * Hp / e);
    out.aV = P.ks * cstr / (e * e);
    out.aH = Hd > 0.0 ? -P.kh / e : 0.0;
    if (Ed > 1.0)
      dcorr = P.ks * Vd * ((bi + 0.5) * dbi / (e * e) - 2.0 * cstr / (e * e * e)) + P.kh * Hp / (e * e);
  }
  out.f = double(W) * corr * F;
  out.A = (dlogF + dcorr) * Pk + Cs + out.aV * Cv + out.aH * Ch;
  return out;
}

// Copies the staged FP64 columns into the walk's precision (FP32 instance) or
// uses them in place (FP64 instance).
__device__ __forceinline__ const Real* convert_columns(double* cols, unsigned char* spare, int count) {
  if constexpr (sizeof(Real) == 8) {
    return reinterpret_cast<const Real*>(cols);
  } else {
    Real* out = reinterpret_cast<Real*>(spare);
    for (int i = threadIdx.x; i < count; i += blockDim.x) out[i] = Real(cols[i]);
    __syncthreads();
    return out;
  }
}

__global__ void __launch_bounds__(kThreads) wtomo_kernel(const __grid_constant__ Params P) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  double* cols = reinterpret_cast<double*>(smem + 16);
  if (!stage_columns(cols, P.col, wt::kSlots, P.col_bytes, bar, P.wait_iters)) {
    if (threadIdx.x == 0) atomicExch(P.err_flag, 1);
    return;
  }
  const int ld = int(P.col_bytes / 8);
  const Real* base = convert_columns(cols, smem + 16 + size_t(wt::kSlots) * P.col_bytes,
                                     wt::kSlots * ld);
  Tables tb;
#pragma unroll
  for (int s = 0; s < wt::kSlots; ++s) tb.c[s] = base + size_t(s) * ld;
  tb.n = P.tv.n;
  tb.uniform = P.tv.uniform;
  tb.lE0 = Real(P.tv.lE0);
  tb.inv_dlE = Real(P.tv.inv_dlE);
  const Consts k{Real(P.mass), Real(P.ctau), Real(P.rho_rock), Real(P.rho_water),
                 Real(P.rho_porous), Real(P.det_elev)};

  const int lane = threadIdx.x & 31;
  const int n_chunks = (P.n_e + 31) / 32;
  // bins are handed out one at a time as warps finish (path lengths differ
  // widely; a static stride leaves a partial last round)
  auto next_bin = [&]() -> long {
    unsigned long long v = 0;
    if (lane == 0) v = atomicAdd(P.next_bin, 1ull);
    return long(__shfl_sync(0xffffffffu, v, 0));
  };
  for (long b = next_bin(); b < P.n_bins; b = next_bin()) {
    const int64_t s0 = P.seg_ptr[b], s1 = P.seg_ptr[b + 1];
    const double ct = P.cos_t[b];
    // device-array calls: cells outside the water-fraction vector end the call
    bool bad = false;
    for (int64_t j = s0 + lane; j < s1; j += 32) bad |= P.seg_cell[j] < 0 || P.seg_cell[j] >= P.n_cells;
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
        for (int64_t j = s0 + lane; j < s1; j += 32) P.jac[j] = 0.0;
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
        L[ch] = pass1(P, k, tb, b, P.E[s], P.q[s]);
        L[ch].f *= 2.0 * P.ew[s];
      }
      sum += L[ch].f;
    }
    sum = wt::warp_sum(sum);
    // geometric and material multipliers (:405-412, :557-579), FP64
    double Lsum = 0.0, water = 0.0, mass = 0.0;
    for (int64_t j = s0 + lane; j < s1; j += 32) {
      const int cell = P.seg_cell[j];
      const double gx = P.seg_len[j] * wt::density64(P, cell);
      Lsum += P.seg_len[j];
      water += P.wf[cell] * gx;
      mass += gx;
    }
    Lsum = wt::warp_sum(Lsum);
    water = wt::warp_sum(water);
    mass = wt::warp_sum(mass) + P.rem[b] * P.rho_rock;
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
      Real E = active ? Real(P.E[s]) : Real(0);
      double Pk = 1.0, Cs = 0.0, Cv = 0.0, Ch = 0.0;
      bool alive = active;
      for (int64_t j = s0; j < s1; ++j) {
        double gk = 0.0;
        if (alive) {
          const int cell = P.seg_cell[j];
          Cell<2> c{seed<2>(Real(P.wf[cell]), 1), wt::cell_porous(P, cell)};
          T<2> rho = cell_density(k, c);
          T<2> e = seed<2>(E, 0), g = cst<2>(Real(1));
          const T<2> e_in = e;
          const Real len = Real(P.seg_len[j]);
          if (solid_segment(k, [&](T<2> x) { return cell_S(tb, c, x); }, rho, len, e, g)) {
            T<2> v, h;
            vh_cell(tb, c, Real(0.5) * (e_in + e), len * rho, v, h);
            Cs += double(g.d[0] / g.v) * Pk;
            Cv += double(v.d[0]) * Pk;
            Ch += double(h.d[0]) * Pk;
            Pk *= double(e.d[0]);
            const double lam = (l.A - Cs - l.aV * Cv - l.aH * Ch) / Pk;
            gk = l.f * (lam * double(e.d[1]) + double(g.d[1] / g.v) + l.aV * double(v.d[1]) +
                        l.aH * double(h.d[1]));
            E = e.v;
          } else {
            alive = false;  // not reached: pass 1 saw the same valid walk
          }
        }
        gk = wt::warp_sum(gk);
        if (lane == 0) P.jac[j] = (ch ? P.jac[j] : 0.0) + scale * gk;
      }
    }
    // d M / d w through the column water fraction q (:557-579)
    if (P.mcorr) {
      const double dlogM = P.lin + 2.0 * P.quad * qf, mm = fmax(mass, 1e-30);
      __syncwarp();
      for (int64_t j = s0 + lane; j < s1; j += 32) {
        const int cell = P.seg_cell[j];
        double dgx;
        const double gx = P.seg_len[j] * wt::density64(P, cell, &dgx);
        dgx *= P.seg_len[j];
        const double dwater = gx + P.wf[cell] * dgx;
        const double dq = mass > 1e-30 ? (dwater * mm - water * dgx) / (mm * mm) : dwater / mm;
        P.jac[j] += flux * dlogM * dq;
      }
    }
  }
}

}  // namespace WT_NS
}  // namespace dp

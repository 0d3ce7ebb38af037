// wtomo.cpp -- oracle restatement of the water-fraction CSDA forward model of
// src/Tomography.jl (compute_directional_flux_csda / _directional_flux_core,
// :444-820) with its correction multipliers (:85-214, :367-412, :557-579).
// Generic over double and Dual: the derivative with respect to one cell's
// water fraction is the forward-mode tangent of the same discrete program,
// which the reference's segment rules (src/Tomography_rules.jl:33-106) and
// Zygote compute.  TEST INFRASTRUCTURE ONLY.
#include "wtomo.hpp"

#include <algorithm>
#include <cmath>

namespace orc {

namespace {

constexpr double MAX_GAIN = 0.02;    // CSDA_MAX_RELATIVE_GAIN (src/Tomography.jl:89)
constexpr double MAX_STEP_M = 60.0;  // CSDA_MAX_STEP_M (src/Tomography.jl:90)

template <class T> T lookup(const MaterialTable& tb, const std::vector<double>& ys, T E) {
  return interp_fast(E, log(E), tb.E, tb.logE, ys);
}
template <class T> T S_csda(const Physics& p, int m, T E) { return lookup(p.t[m], p.t[m].csda_S, E); }
template <class T> T S_mixed(const Physics& p, int m, T E) { return lookup(p.t[m], p.t[m].mixed_S, E); }
template <class T> T omega(const Physics& p, int m, T E) { return lookup(p.t[m], p.t[m].strag, E); }

bool porous(bool shallow, const WConfig& c) {  // is_shallow_porous, :299-301
  return shallow && c.porous >= 0 && c.porous_top > 0.0;
}

// cell_density / cell_stopping_power / cell_straggling / cell_hardloss (:303-352)
template <class T> T cell_density(T w, bool sh, const WConfig& c) {
  if (porous(sh, c))
    return T(1.0) / (T(0.5) * (T(1.0) - w) / T(c.rho_porous) + T(0.5) * (T(1.0) - w) / T(c.rho_rock) +
                     w / T(c.rho_water));
  return T(1.0) / ((T(1.0) - w) / T(c.rho_rock) + w / T(c.rho_water));
}
template <class T, class F> T cell_mix(T w, bool sh, const WConfig& c, F prop) {
  if (porous(sh, c))
    return T(0.5) * (T(1.0) - w) * prop(c.porous) + T(0.5) * (T(1.0) - w) * prop(c.rock) +
           w * prop(c.water);
  return (T(1.0) - w) * prop(c.rock) + w * prop(c.water);
}
template <class T> T cell_S(const Physics& p, T w, bool sh, const WConfig& c, T E) {
  return cell_mix(w, sh, c, [&](int m) { return S_csda(p, m, E); });
}
template <class T> T cell_omega(const Physics& p, T w, bool sh, const WConfig& c, T E) {
  return cell_mix(w, sh, c, [&](int m) { return omega(p, m, E); });
}
template <class T> T cell_hard(const Physics& p, T w, bool sh, const WConfig& c, T E) {
  // the porous term is used only in the porous top layer (:341-352)
  return cell_mix(w, sh, c, [&](int m) { return S_csda(p, m, E) - S_mixed(p, m, E); });
}

// compute_decay_weight_from_path (src/Geometry.jl:1083-1107)
template <class T> T decay(const Physics& p, T L, T Eavg) {
  T g = T(1.0) + Eavg / T(p.mass);
  T b2 = T(1.0) - T(1.0) / (g * g);
  T b = sqrt(val(b2) >= 1e-12 ? b2 : T(1e-12));
  return exp(-L / (b * g * T(p.ctau)));
}

// The Heun step shared by the three propagators (:455-471): returns false on
// an invalid step (weight set to zero).
template <class T, class SFun>
bool heun(const Physics& p, SFun S, T dedx0, T ds, T density, T& E, T& W) {
  T grammage = ds * density;
  T Ep = E + dedx0 * grammage;
  T dedx1 = S(Ep);
  T dE = T(0.5) * (dedx0 + dedx1) * grammage;
  T En = E + dE;
  if (!isfinite(En) || val(En) >= 1e12) {
    E = En;
    W = T(0.0);
    return false;
  }
  T dedxn = S(En);
  W = W * (dedxn / jmax(dedx0, T(1e-30)));
  W = W * decay(p, ds, T(0.5) * (E + En));
  E = En;
  return true;
}

// propagate_csda_cell_segment / propagate_csda_uniform_segment (:444-509)
template <class T, class SFun>
bool solid_segment(const Physics& p, SFun S, T density, double distance, T& E, T& W) {
  T remaining = T(distance);
  while (val(remaining) > 1e-8) {
    T dedx0 = S(E);
    if (!isfinite(dedx0) || val(dedx0) <= 0.0) {
      W = T(0.0);
      return false;
    }
    T grel = T(MAX_GAIN) * jmax(E, T(1e-6)) / dedx0;
    T gstep = jmin(jmin(remaining * density, jmax(grel, T(1e-6))), T(MAX_STEP_M) * density);
    T ds = jmin(remaining, gstep / jmax(density, T(1e-12)));
    if (val(ds) <= 0.0) {
      W = T(0.0);
      return false;
    }
    if (!heun(p, S, dedx0, ds, density, E, W)) return false;
    remaining = remaining - ds;
  }
  return true;
}

// propagate_csda_air_segment (:516-551)
template <class T>
bool air_segment(const Physics& p, const WConfig& c, double start_z, double cos_t,
                 double distance, T& E, T& W) {
  // remaining and traversed carry the tangent of the steps, and with them the
  // altitude of the density (the reference's values become duals once a step does)
  auto S = [&](T e) { return S_csda(p, c.air, e); };
  T remaining = T(distance), traversed = T(0.0);
  const T base = T(c.det_elev + start_z);
  while (val(remaining) > 1e-8) {
    T alt = base + T(cos_t) * (traversed + T(0.5) * jmin(remaining, T(MAX_STEP_M)));
    T rho = T(1.205) * exp(-alt / T(12e3));
    T dedx0 = S(E);
    if (!isfinite(dedx0) || val(dedx0) <= 0.0) {
      W = T(0.0);
      return false;
    }
    T grel = T(MAX_GAIN) * jmax(E, T(1e-6)) / dedx0;
    T ds = jmin(jmin(remaining, T(MAX_STEP_M)), grel / jmax(rho, T(1e-12)));
    ds = jmax(ds, T(1e-3));
    alt = base + T(cos_t) * (traversed + T(0.5) * ds);
    rho = T(1.205) * exp(-alt / T(12e3));
    if (!heun(p, S, dedx0, ds, rho, E, W)) return false;
    traversed = traversed + ds;
    remaining = remaining - ds;
  }
  return true;
}

// flux_gccly charge +1 at E (1 +- eta) for the local spectral index (:367-372)
template <class T> T spectral_index(T E, double cos_t) {
  const double eta = 1e-2;
  T fp = flux_gccly(cos_t, E * T(1.0 + eta), 1.0);
  T fm = flux_gccly(cos_t, E * T(1.0 - eta), 1.0);
  return -(log(fp) - log(fm)) / T(2 * eta);
}
double spectral_index(double E, double cos_t) { return spectral_index<double>(E, cos_t); }

// csda_var_correction (:384-391)
template <class T> T var_correction(const WConfig& c, T Es, T V, T H, double cos_t) {
  if (!c.corr) return T(1.0);
  T e = jmax(Es, T(1.0));
  T b = spectral_index(e, cos_t);
  T cs = T(0.5) * b * (b + T(1.0));
  return exp(T(c.ks) * cs * V / (e * e) - T(c.kh) * jmax(H, T(0.0)) / e);
}

}  // namespace

// _directional_flux_core / compute_directional_flux_csda (:580-727) for one
// path; w holds the water fraction of every cell (as T).
template <class T>
T dir_flux_csda(const Physics& p, const WConfig& c, const WPath& path, const unsigned char* shallow,
                const T* w, const double* E, const double* q, const double* ew, int n_e) {
  if (!path.valid || !(path.cos_theta > 0.0)) return T(NAN);
  const double ct = path.cos_theta;
  T sum = T(0.0);
  for (int s = 0; s < n_e; ++s) {
    T energy = T(E[s]), weight = T(1.0), V = T(0.0), H = T(0.0);
    bool ok = true;
    for (long k = 0; k < path.n_seg; ++k) {
      const int cell = path.cell[k];
      const bool sh = shallow && shallow[cell];
      T wk = w[cell];
      T rho = cell_density(wk, sh, c);
      T e_in = energy;
      ok = solid_segment(p, [&](T e) { return cell_S(p, wk, sh, c, e); }, rho, path.len[k], energy,
                         weight);
      if (!ok) break;
      T e_rep = T(0.5) * (e_in + energy);
      T gx = T(path.len[k]) * rho;
      V = V + cell_omega(p, wk, sh, c, e_rep) * gx;
      H = H + cell_hard(p, wk, sh, c, e_rep) * gx;
    }
    if (ok && path.remaining_rock > 1e-8) {
      T e_in = energy;
      ok = solid_segment(p, [&](T e) { return S_csda(p, c.rock, e); }, T(c.rho_rock),
                         path.remaining_rock, energy, weight);
      if (ok) {
        T e_rep = T(0.5) * (e_in + energy);
        T gx = T(path.remaining_rock * c.rho_rock);
        V = V + omega(p, c.rock, e_rep) * gx;
        H = H + (S_csda(p, c.rock, e_rep) - S_mixed(p, c.rock, e_rep)) * gx;
      }
    }
    if (ok) {
      double air = std::max(0.0, c.primary - path.exit_z) / std::max(ct, 1e-3);
      ok = air_segment(p, c, path.exit_z, ct, air, energy, weight);
    }
    T fs = T(0.0);
    if (ok) fs = weight * var_correction(c, energy, V, H, ct) * flux_gccly(ct, energy, q[s]);
    sum = sum + T(2.0 * ew[s]) * fs;
  }
  // geometric and material multipliers (:405-412, :557-579)
  T mult = T(1.0);
  if (c.corr && (c.ra != 0.0 || c.rb != 0.0 || c.rc != 0.0 || c.rd != 0.0)) {
    double L = path.remaining_rock;
    for (long k = 0; k < path.n_seg; ++k) L += path.len[k];
    double lL = std::log(std::max(L, 1.0));
    mult = T(std::exp(c.ra + c.rb * lL + c.rc * lL * lL + c.rd * ct));
  }
  if (c.mcorr) {
    T water = T(0.0), mass = T(path.remaining_rock * c.rho_rock);
    for (long k = 0; k < path.n_seg; ++k) {
      const int cell = path.cell[k];
      T gx = T(path.len[k]) * cell_density(w[cell], shallow && shallow[cell], c);
      water = water + w[cell] * gx;
      mass = mass + gx;
    }
    T qf = water / jmax(mass, T(1e-30));
    mult = mult * exp(T(c.lin) * qf + T(c.quad) * qf * qf);
  }
  return mult * sum / T(double(n_e));
}

template double dir_flux_csda<double>(const Physics&, const WConfig&, const WPath&,
                                      const unsigned char*, const double*, const double*,
                                      const double*, const double*, int);
template Dual dir_flux_csda<Dual>(const Physics&, const WConfig&, const WPath&,
                                  const unsigned char*, const Dual*, const double*, const double*,
                                  const double*, int);

}  // namespace orc

// transport.cpp -- oracle restatement of the deterministic CSDA transport
// (src/Geometry.jl), the surface spectrum (src/GaisserFlux.jl) and the
// voxel-density tomography forward model (examples/diff_flux_cube.jl).
// Templated on double and Dual so one code path yields values and the exact
// derivative of the discrete program.  TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <limits>

#include "oracle.hpp"

namespace orc {

template <class T> static T jpow(T x, double a) { return exp(T(a) * log(x)); }
static double jpow(double x, double a) { return std::pow(x, a); }

// ------------------------------------------------------------ GaisserFlux
// src/GaisserFlux.jl:62-76
double cos_theta_star(double c) {
  const double p0 = 0.102573, p1 = -0.068287, p2 = 0.958633, p3 = 0.0407253, p4 = 0.817285;
  double cs2 = (c * c + p0 * p0 + p1 * std::pow(c, p2) + p3 * std::pow(c, p4)) /
               (1.0 + p0 * p0 + p1 + p3);
  return cs2 > 0 ? std::sqrt(cs2) : 0.0;
}
// src/GaisserFlux.jl:93-105
template <class T> static T gaisser(double c, T K, double q) {
  T Emu = K + T(MUON_MASS);
  T ec = T(1.1) * Emu * T(c);
  T rpi = T(1.0) + ec / T(115.0);
  T rK = T(1.0) + ec / T(850.0);
  return T(1.4e3) * jpow(Emu, -2.7) * (T(1.0) / rpi + T(0.054) / rK) * charge_fraction(T(q));
}
// src/GaisserFlux.jl:125-133
template <class T> static T gccly(double c, T K, double q) {
  T Emu = K + T(MUON_MASS);
  double cs = cos_theta_star(c);
  T f = jpow(T(1.0) + T(3.64) / (Emu * T(std::pow(cs, 1.29))), -2.7);
  return f * gaisser(cs, K, q);
}
double flux_gaisser(double c, double K, double q) { return gaisser<double>(c, K, q); }
double flux_gccly(double c, double K, double q) { return gccly<double>(c, K, q); }
Dual flux_gccly(double c, Dual K, double q) { return gccly<Dual>(c, K, q); }

// ------------------------------------------------------------ CSDA step
// src/Geometry.jl:1083-1093
template <class T> static T decay_from_path(const Physics& p, T L, T Eavg) {
  T g = T(1.0) + Eavg / T(p.mass);
  T b = sqrt(jmax(T(1.0) - T(1.0) / (g * g), T(1e-12)));
  return exp(-L / (b * g * T(p.ctau)));
}

template <class T> struct CState {
  T E, w, z, t;
};

// src/Geometry.jl:424-457 (transport_backward_step, rng = nothing)
template <class T>
static void csda_step(const Physics& p, CState<T>& s, const MaterialTable& tb, T density,
                      T step, double dir_z) {
  T ki = s.E;
  T dX = step * density;
  T Xi = csda_range(tb, ki);
  T kf = csda_energy(tb, Xi + dX);
  T gi = T(1.0) + ki / T(p.mass), gc = T(1.0) + kf / T(p.mass), ga = (gi + gc) / T(2.0);
  T ba = sqrt(jmax(T(1.0) - T(1.0) / (ga * ga), T(1e-12)));
  T dt = step / (ba * ga);
  s.z = s.z - step * T(dir_z);
  T Si = csda_stopping(tb, ki), Sf = csda_stopping(tb, kf);
  s.w = s.w * (Sf / Si) * exp(-dt / T(p.ctau));
  s.t = s.t + dt;
  s.E = kf;
}

// src/Geometry.jl:461-476
template <class T>
static T geometric_limit(const Physics& p, const MaterialTable& tb, T E, T density, double uz,
                         bool in_air, bool use_scattering) {
  const double inf = std::numeric_limits<double>::infinity();
  T Xi = csda_range(tb, E);
  T range_limit = T(0.01) * Xi / jmax(density, T(1e-6));
  T scat_limit = T(inf);
  if (use_scattering) {
    T lb1 = interp_fast(E, log(E), tb.E, tb.logE, tb.lb1);
    if (val(lb1) > 0 && val(density) > 0) scat_limit = T(0.01) * lb1 / density;
  }
  T air_limit = in_air ? T(0.05 * 12e3 / std::max(std::fabs(uz), 0.05)) : T(inf);
  return jmin(jmin(range_limit, scat_limit), air_limit);
}

// src/Geometry.jl:534-672 (transport_backward_through_geometry, rng = nothing)
// followed by the acceptance of src/Geometry.jl:694-757.
template <class T>
T flux_single_csda(const Physics& p, const TwoLayer& g, T rho, double elevation,
                   double energy, double charge, double threshold, long* steps_out) {
  double theta = (90.0 - elevation) * PI / 180.0;
  double cth = std::cos(theta), sth = std::sin(theta);
  (void)sth;
  double dir_z = -cth;
  CState<T> s{T(energy), T(1.0), T(0.0), T(0.0)};
  const double low = 100.0, eps = EPS64, H = g.primary_altitude;
  long steps = 0;
  for (int outer = 0; outer < 1000000 && val(s.E) < threshold - eps; ++outer) {
    double z = val(s.z);
    if (z < 0) break;
    if (z >= H - eps) break;
    if (val(s.w) <= 0 || !isfinite(s.w)) break;
    double limit = val(s.E) < low - eps ? std::min(low, threshold) : threshold;
    bool use_scat = false;  // scattering=false on the deterministic path
    for (int inner = 0; inner < 50000; ++inner) {
      double zv = val(s.z);
      if (zv < 0 || zv >= H - eps) break;
      if (val(s.E) >= limit - eps) break;
      if (val(s.w) <= 0 || !isfinite(s.w)) break;
      double uz = -dir_z;
      const MaterialTable* tb;
      T density, to_boundary;
      bool in_air = zv >= g.thickness;
      if (!in_air) {
        tb = &p.t[g.rock];
        density = rho;
        if (uz > eps) to_boundary = (T(g.thickness) - s.z) / T(uz);
        else if (uz < -eps) to_boundary = (T(0.0) - s.z) / T(uz);
        else to_boundary = T(1000.0);
      } else {
        tb = &p.t[g.air];
        density = T(1.205) * exp(-s.z / T(12e3));
        if (uz > eps) to_boundary = (T(H) - s.z) / T(uz);
        else if (uz < -eps) to_boundary = (T(g.thickness) - s.z) / T(uz);
        else to_boundary = T(1000.0);
      }
      T lim = geometric_limit(p, *tb, s.E, density, uz, in_air, use_scat);
      T step = jmin(to_boundary + T(1e-7), lim);
      // clamp(x, lo, hi)
      if (val(step) < STEP_MIN) step = T(STEP_MIN);
      else if (val(step) > 1000.0) step = T(1000.0);
      csda_step(p, s, *tb, density, step, dir_z);
      ++steps;
    }
  }
  if (steps_out) *steps_out = steps;
  if (val(s.z) >= H - 1.0 && val(s.E) < threshold) {
    double c = std::min(std::max(-dir_z, 0.0), 1.0);
    if (c <= 0) return T(0.0);
    return s.w * gccly<T>(c, s.E, charge);
  }
  return T(0.0);
}
template double flux_single_csda<double>(const Physics&, const TwoLayer&, double, double,
                                         double, double, double, long*);
template Dual flux_single_csda<Dual>(const Physics&, const TwoLayer&, Dual, double, double,
                                     double, double, long*);

// src/Geometry.jl:1043-1055
template <class T> static T air_grammage(double z0, double z1, double c) {
  double cs = std::max(std::fabs(c), 0.01);
  double g = (1.205 * 12e3 / cs) * (std::exp(-z0 / 12e3) - std::exp(-z1 / 12e3));
  return T(std::max(g, 0.0));
}

// src/Geometry.jl:1126-1209
template <class T>
T flux_csda_direct(const Physics& p, int rock, int air, T rho, double thickness,
                   double elevation, double energy, double charge, double H) {
  double el = elevation * (PI / 180.0);
  double c = std::cos(PI / 2 - el);
  double cs = std::max(std::fabs(c), 0.01);
  const MaterialTable &tr = p.t[rock], &ta = p.t[air];
  T Xr = T(thickness / cs) * rho;
  T E0 = T(energy);
  T E1 = csda_energy(tr, csda_range(tr, E0) + Xr);
  if (val(E1) >= 1e12 || !isfinite(E1)) return T(0.0);
  T wr = csda_stopping(tr, E1) / csda_stopping(tr, E0);
  T dr = decay_from_path(p, T(thickness / cs), (E0 + E1) / T(2.0));
  T Xa = air_grammage<T>(thickness, H, c);
  T E2 = csda_energy(ta, csda_range(ta, E1) + Xa);
  if (val(E2) >= 1e12 || !isfinite(E2)) return T(0.0);
  T wa = csda_stopping(ta, E2) / csda_stopping(ta, E1);
  T da = decay_from_path(p, T((H - thickness) / cs), (E1 + E2) / T(2.0));
  return wr * dr * wa * da * gccly<T>(c, E2, charge);
}
template double flux_csda_direct<double>(const Physics&, int, int, double, double, double,
                                         double, double, double);
template Dual flux_csda_direct<Dual>(const Physics&, int, int, Dual, double, double, double,
                                     double, double);

// ------------------------------------------------------------ tomography
// examples/diff_flux_cube.jl:132-148
static bool cell_of(const Grid& g, double x, double y, double z, int& i, int& j, int& k) {
  double xmax = g.x0 + g.nx * g.dx, ymax = g.y0 + g.ny * g.dy, zmax = g.z0 + g.nz * g.dz;
  if (x < g.x0 || x > xmax || y < g.y0 || y > ymax || z < g.z0 || z > zmax) return false;
  i = std::min(std::max(int(std::floor((x - g.x0) / g.dx)) + 1, 1), g.nx);
  j = std::min(std::max(int(std::floor((y - g.y0) / g.dy)) + 1, 1), g.ny);
  k = std::min(std::max(int(std::floor((z - g.z0) / g.dz)) + 1, 1), g.nz);
  return true;
}

// examples/diff_flux_cube.jl:194-298 (distance to the next cell boundary,
// candidates tested x then y then z with strict improvement)
static double to_boundary(const Grid& g, double x, double y, double z, double ux, double uy,
                          double uz, bool& exiting) {
  int i, j, k;
  exiting = true;
  if (!cell_of(g, x, y, z, i, j, k)) return 0.0;
  double xlo = g.x0 + (i - 1) * g.dx, xhi = g.x0 + i * g.dx;
  double ylo = g.y0 + (j - 1) * g.dy, yhi = g.y0 + j * g.dy;
  double zlo = g.z0 + (k - 1) * g.dz, zhi = g.z0 + k * g.dz;
  double tmin = std::numeric_limits<double>::infinity();
  const double eps = 1e-10;
  exiting = false;
  if (std::fabs(ux) > eps) {
    double t = ux > 0 ? (xhi - x) / ux : (xlo - x) / ux;
    if (t > eps && t < tmin) {
      tmin = t;
      exiting = ux > 0 ? (i + 1 > g.nx) : (i - 1 < 1);
    }
  }
  if (std::fabs(uy) > eps) {
    double t = uy > 0 ? (yhi - y) / uy : (ylo - y) / uy;
    if (t > eps && t < tmin) {
      tmin = t;
      exiting = uy > 0 ? (j + 1 > g.ny) : (j - 1 < 1);
    }
  }
  if (std::fabs(uz) > eps) {
    double t = uz > 0 ? (zhi - z) / uz : (zlo - z) / uz;
    if (t > eps && t < tmin) {
      tmin = t;
      exiting = uz > 0 ? (k + 1 > g.nz) : (k - 1 < 1);
    }
  }
  if (tmin == std::numeric_limits<double>::infinity()) exiting = true;
  return tmin;
}

// examples/diff_flux_cube.jl:304-366 (trace_cube_path)
RayTrace trace_ray(const Grid& g, const Ray& r) {
  RayTrace tr;
  double x = r.ox, y = r.oy, z = r.oz;
  tr.z_exit = z;
  for (int step = 0; step < 1000; ++step) {
    int i, j, k;
    if (!cell_of(g, x, y, z, i, j, k)) break;
    int cell = (i - 1) + g.nx * ((j - 1) + g.ny * (k - 1));
    bool exiting;
    double d = to_boundary(g, x, y, z, r.ux, r.uy, r.uz, exiting);
    if (d <= 1e-10 || !std::isfinite(d)) {
      x += r.ux * 0.01;
      y += r.uy * 0.01;
      z += r.uz * 0.01;
      continue;
    }
    tr.seg.push_back({cell, d});
    x += r.ux * d;
    y += r.uy * d;
    z += r.uz * d;
    tr.z_exit = z;
    if (exiting) break;
  }
  return tr;
}

// examples/diff_flux_cube.jl:374-470 (compute_flux_from_segments), with the
// side-exit remainder density as an explicit input and the primary altitude
// as a parameter.
template <class T>
static bool csda_segment(const Physics& p, const MaterialTable& tb, T& E, T& w, T rho, double L) {
  T Xi = csda_range(tb, E);
  T Ea = csda_energy(tb, Xi + T(L) * rho);
  if (val(Ea) >= 1e12 || !isfinite(Ea)) return false;
  w = w * (csda_stopping(tb, Ea) / csda_stopping(tb, E));
  w = w * decay_from_path(p, T(L), (E + Ea) / T(2.0));
  E = Ea;
  return true;
}
template <class T>
T tomo_flux_node(const Physics& p, int rock, int air, const Grid& g, const RayTrace& tr,
                 double cos_theta, const double* rho, double rho_side, int seed, double energy,
                 double charge, double H) {
  const MaterialTable &trk = p.t[rock], &ta = p.t[air];
  T E = T(energy), w = T(1.0);
  for (const Segment& s : tr.seg) {
    T d = T(rho[s.cell], s.cell == seed ? 1.0 : 0.0);
    if (!csda_segment(p, trk, E, w, d, s.len)) return T(0.0);
  }
  double zmax = g.z0 + g.nz * g.dz;
  if (tr.z_exit < zmax - EPS64) {
    double cs = std::max(std::fabs(cos_theta), 0.01);
    double L = (zmax - tr.z_exit) / cs;
    T d = T(rho_side, seed == -2 ? 1.0 : 0.0);
    if (!csda_segment(p, trk, E, w, d, L)) return T(0.0);
  }
  T Xa = air_grammage<T>(zmax, H, cos_theta);
  T Ef = csda_energy(ta, csda_range(ta, E) + Xa);
  if (val(Ef) >= 1e12 || !isfinite(Ef)) return T(0.0);
  w = w * (csda_stopping(ta, Ef) / csda_stopping(ta, E));
  double cs = std::max(std::fabs(cos_theta), 0.01);
  w = w * decay_from_path(p, T((H - zmax) / cs), (E + Ef) / T(2.0));
  return w * gccly<T>(cos_theta, Ef, charge);
}
template <>
double tomo_flux_node<double>(const Physics& p, int rock, int air, const Grid& g,
                              const RayTrace& tr, double cos_theta, const double* rho,
                              double rho_side, int, double energy, double charge, double H) {
  const MaterialTable &trk = p.t[rock], &ta = p.t[air];
  double E = energy, w = 1.0;
  for (const Segment& s : tr.seg)
    if (!csda_segment<double>(p, trk, E, w, rho[s.cell], s.len)) return 0.0;
  double zmax = g.z0 + g.nz * g.dz;
  if (tr.z_exit < zmax - EPS64) {
    double cs = std::max(std::fabs(cos_theta), 0.01);
    if (!csda_segment<double>(p, trk, E, w, rho_side, (zmax - tr.z_exit) / cs)) return 0.0;
  }
  double Xa = air_grammage<double>(zmax, H, cos_theta);
  double Ef = csda_energy(ta, csda_range(ta, E) + Xa);
  if (Ef >= 1e12 || !std::isfinite(Ef)) return 0.0;
  w *= csda_stopping(ta, Ef) / csda_stopping(ta, E);
  double cs = std::max(std::fabs(cos_theta), 0.01);
  w *= decay_from_path<double>(p, (H - zmax) / cs, (E + Ef) / 2.0);
  return w * gccly<double>(cos_theta, Ef, charge);
}
template Dual tomo_flux_node<Dual>(const Physics&, int, int, const Grid&, const RayTrace&,
                                   double, const double*, double, int, double, double, double);

// Reverse-mode derivative of tomo_flux_node with respect to every segment
// density (the side-exit remainder last), by a backward sweep over the stored
// forward energies -- the CPU counterpart of the GPU adjoint, used to time the
// CPU baseline of forward + adjoint.  Returns the flux; dseg gets one entry per
// segment (+1 if there is a side-exit remainder).
double tomo_node_adjoint(const Physics& p, int rock, int air, const Grid& g, const RayTrace& tr,
                         double cos_theta, const double* rho, double rho_side, double energy,
                         double charge, double H, std::vector<double>& dseg) {
  const MaterialTable &trk = p.t[rock], &ta = p.t[air];
  double zmax = g.z0 + g.nz * g.dz;
  double cs = std::max(std::fabs(cos_theta), 0.01);
  size_t ns = tr.seg.size();
  bool side = tr.z_exit < zmax - EPS64;
  size_t nt = ns + (side ? 1 : 0);
  std::vector<double> L(nt), D(nt), E(nt + 1);
  for (size_t s = 0; s < ns; ++s) {
    L[s] = tr.seg[s].len;
    D[s] = rho[tr.seg[s].cell];
  }
  if (side) {
    L[ns] = (zmax - tr.z_exit) / cs;
    D[ns] = rho_side;
  }
  dseg.assign(nt, 0.0);
  // forward, with the derivative of each step's map E -> E' recorded
  E[0] = energy;
  double w = 1.0;
  for (size_t s = 0; s < nt; ++s) {
    double Ea = csda_energy(trk, csda_range(trk, E[s]) + L[s] * D[s]);
    if (Ea >= 1e12 || !std::isfinite(Ea)) return 0.0;
    w *= csda_stopping(trk, Ea) / csda_stopping(trk, E[s]);
    w *= decay_from_path<double>(p, L[s], (E[s] + Ea) / 2.0);
    E[s + 1] = Ea;
  }
  double EN = E[nt];
  double Ga = air_grammage<double>(zmax, H, cos_theta);
  Dual ENd(EN, 1.0);
  Dual Ef = csda_energy(ta, csda_range(ta, ENd) + Dual(Ga));
  if (Ef.v >= 1e12 || !std::isfinite(Ef.v)) return 0.0;
  // d log(air factor * flux)/d EN through duals seeded on EN, plus the rock
  // stopping power of the last segment
  Dual La = Dual((H - zmax) / cs);
  Dual logA = log(csda_stopping(ta, Ef)) - log(csda_stopping(ta, ENd)) +
              log(decay_from_path<Dual>(p, La, (ENd + Ef) / Dual(2.0))) +
              log(gccly<Dual>(cos_theta, Ef, charge));
  double flux = w * std::exp(logA.v);
  double lam = logA.d + csda_stopping(trk, Dual(EN, 1.0)).d / csda_stopping(trk, EN);
  for (size_t s = nt; s-- > 0;) {
    // E_{s+1} = K(R(E_s) + L D): derivatives by duals at the stored point
    Dual Es(E[s], 1.0);
    Dual Y = csda_range(trk, Es) + Dual(L[s] * D[s]);
    Dual Ey = csda_energy(trk, Dual(Y.v, 1.0));    // dE'/dY
    Dual Ee = csda_energy(trk, Y);                  // dE'/dE_s
    Dual Da = log(decay_from_path<Dual>(p, Dual(L[s]), (Dual(E[s]) + Dual(E[s + 1], 1.0)) / Dual(2.0)));
    Dual Db = log(decay_from_path<Dual>(p, Dual(L[s]), (Es + Dual(E[s + 1])) / Dual(2.0)));
    lam += Da.d;
    dseg[s] = flux * lam * Ey.d * L[s];
    lam = lam * Ee.d + Db.d;
  }
  return flux;
}

}  // namespace orc

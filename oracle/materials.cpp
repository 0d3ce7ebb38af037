// materials.cpp -- oracle restatement of src/Materials.jl (elements, atomic
// shells, Fano density effect, electronic stopping, SSR/DRSS/Salvat DCS and
// their log-scale Gauss-Legendre moments).  TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <map>
#include <stdexcept>

#include "oracle.hpp"
#include "physics_data.inc"

namespace orc {

// ------------------------------------------------------------ elements
// src/Materials.jl:35-48
const Element& element(const std::string& s) {
  static const std::map<std::string, Element> tab = {
      {"H", {"H", 1.0, 1.00794, 19.2e-9}},   {"C", {"C", 6.0, 12.0107, 78.0e-9}},
      {"N", {"N", 7.0, 14.0067, 82.0e-9}},   {"O", {"O", 8.0, 15.9994, 95.0e-9}},
      {"Na", {"Na", 11.0, 22.9898, 149.0e-9}}, {"Mg", {"Mg", 12.0, 24.305, 156.0e-9}},
      {"Al", {"Al", 13.0, 26.9815, 166.0e-9}}, {"Si", {"Si", 14.0, 28.0855, 173.0e-9}},
      {"K", {"K", 19.0, 39.0983, 190.0e-9}},  {"Ca", {"Ca", 20.0, 40.078, 191.0e-9}},
      {"Fe", {"Fe", 26.0, 55.845, 286.0e-9}}, {"Ar", {"Ar", 18.0, 39.948, 188.0e-9}},
  };
  auto it = tab.find(s);
  if (it == tab.end()) throw std::runtime_error("unknown element " + s);
  return it->second;
}

// src/Materials.jl:50-66 (BaseMaterial constructor normalises and forms Z/A)
BaseMaterial make_material(const std::string& name, double density, double I,
                           const std::vector<Element>& els, const std::vector<double>& fr) {
  BaseMaterial m;
  m.name = name;
  m.density = density;
  m.I = I;
  m.elements = els;
  double tot = 0;
  for (double f : fr) tot += f;
  m.ZoA = 0;
  for (size_t i = 0; i < fr.size(); ++i) {
    m.fractions.push_back(fr[i] / tot);
    m.ZoA += els[i].Z / els[i].A * m.fractions.back();
  }
  return m;
}

// src/Materials.jl:110-127
BaseMaterial standard_rock() {
  return make_material("StandardRock", 2650.0, 136.4e-9,
                       {element("O"), element("Si"), element("Al"), element("Fe"),
                        element("Ca"), element("Na"), element("Mg"), element("K")},
                       {0.466, 0.277, 0.081, 0.050, 0.036, 0.028, 0.021, 0.026});
}
BaseMaterial air() {
  return make_material("Air", 1.205, 85.7e-9, {element("N"), element("O"), element("Ar")},
                       {0.755, 0.232, 0.013});
}
BaseMaterial water() {
  return make_material("Water", 1000.0, 75.0e-9, {element("H"), element("O")},
                       {0.1119, 0.8881});
}

// ------------------------------------------------------------ quadrature
// Gauss-Legendre nodes/weights on [0, 1] by Newton iteration on P_n.  (The
// reference tabulates the same nodes, src/Materials.jl:141-227.)
void gauss_legendre01(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = std::cos(PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-16) break;
    }
    // ascending order on [0, 1]
    x[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z * z) * pp * pp);
  }
}
namespace {
struct GQ {
  double x[12], w[12];
  explicit GQ(int n) { gauss_legendre01(n, x, w); }
};
const GQ& gq(int n) {
  static const GQ g9(9), g12(12);
  return n == 9 ? g9 : g12;
}
}  // namespace

// ------------------------------------------------------------ dilogarithm
// Real dilogarithm Li2(x) (same function as src/Materials.jl:286-339, by our
// own method): the Bernoulli series in u = -log(1-x) on [-1, 1/2] plus the
// standard reflection/inversion identities.
static double li2_series(double x) {
  // Li2(x) = sum_n B_n u^{n+1}/(n+1)!,  u = -log(1-x)
  static const double B[] = {1.0, -0.5, 1.0 / 6, 0, -1.0 / 30, 0, 1.0 / 42, 0, -1.0 / 30,
                             0, 5.0 / 66, 0, -691.0 / 2730, 0, 7.0 / 6, 0, -3617.0 / 510,
                             0, 43867.0 / 798, 0, -174611.0 / 330};
  double u = -std::log1p(-x), s = 0, pw = u, fact = 1;
  for (int n = 0; n <= 20; ++n) {
    fact *= (n + 1);
    if (B[n] != 0) s += B[n] * pw / fact;
    pw *= u;
  }
  return s;
}
double math_dilog(double x) {
  const double pi2_6 = PI * PI / 6;
  if (x == 1.0) return pi2_6;
  if (x == -1.0) return -PI * PI / 12;
  if (x > 1.0) {  // real part
    double l = std::log(x);
    return PI * PI / 3 - 0.5 * l * l - math_dilog(1.0 / x);
  }
  if (x < -1.0) {
    double l = std::log(-x);
    return -pi2_6 - 0.5 * l * l - math_dilog(1.0 / x);
  }
  if (x <= 0.5) {
    if (x >= -1.0) return li2_series(x);
  }
  // 1/2 < x < 1
  return pi2_6 - std::log(x) * std::log1p(-x) - li2_series(1.0 - x);
}

// ------------------------------------------------------------ atomic shells
// src/Materials.jl:360-431
struct Shell {
  double f, E;
};
static void shells_of(int Z, double w, std::vector<Shell>& out) {
  int iZ = std::min(std::max(Z, 1), 100);
  int s0 = DPDATA_SHELL_INDEX[iZ - 1], s1 = DPDATA_SHELL_INDEX[iZ];
  for (int s = s0; s < s1; ++s)
    out.push_back({w * double(DPDATA_SHELL_OCCUPANCY[s]), double(DPDATA_SHELL_ENERGY_EV[s])});
}
static std::vector<Shell> atomic_shells(const BaseMaterial& m) {
  std::vector<Shell> sh;
  for (size_t i = 0; i < m.elements.size(); ++i) {
    const Element& e = m.elements[i];
    double w = m.fractions[i] / e.A;
    if (e.Z == 11.0 && e.A == 22.0) {  // "Rockium": C + 3 O + Ca
      double ws = w * 11.0 / (6.0 + 3 * 8.0 + 20.0);
      shells_of(6, ws, sh);
      shells_of(8, 3 * ws, sh);
      shells_of(20, ws, sh);
    } else {
      shells_of(int(std::lround(e.Z)), w, sh);
    }
  }
  double ftot = 0, lnI = 0;
  for (auto& s : sh) {
    ftot += s.f;
    lnI += s.f * std::log(s.E);
  }
  double inv = 1.0 / ftot;
  lnI *= inv;
  double wp = 28.816 * std::sqrt(m.ZoA * m.density * 1e-3);
  double aS = m.I * 1e9 / std::exp(lnI);
  double r = aS / wp;
  for (auto& s : sh) {
    s.f *= inv;
    s.E *= r;
  }
  return sh;
}

// src/Materials.jl:437-469 (Fano density effect, bisection on l^2)
static double density_effect(const std::vector<Shell>& sh, double gamma) {
  double y = 1.0 / (gamma * gamma), ymax = 0;
  for (auto& s : sh) ymax += s.f / (s.E * s.E);
  if (ymax <= y) return 0.0;
  double l2min = 0, l2max = 1.0 / y, l2 = 0;
  for (int it = 0; it < 200; ++it) {
    l2 = 0.5 * (l2min + l2max);
    double yi = 0;
    for (auto& s : sh) yi += s.f / (s.E * s.E + l2);
    if (std::fabs(yi - y) <= EPS64 || (l2max - l2min) <= EPS64) break;
    if (yi > y) l2min = l2; else l2max = l2;
  }
  double delta = -l2 * y;
  for (auto& s : sh) delta += s.f * std::log(1.0 + l2 / (s.E * s.E));
  return delta;
}

// src/Materials.jl:488-507 (modified Bethe-Bloch with radiative correction)
double electronic_stopping_power(const BaseMaterial& m, double mass, double K) {
  static std::map<std::string, std::vector<Shell>> cache;
  auto it = cache.find(m.name);
  if (it == cache.end()) it = cache.emplace(m.name, atomic_shells(m)).first;
  const auto& sh = it->second;
  double E = K + mass, P2 = K * (K + 2.0 * mass), beta2 = P2 / (E * E), gamma = E / mass;
  double r = ELECTRON_MASS / mass;
  double Qmax = 2.0 * r * P2 / (mass * (1.0 + r * r) + 2.0 * r * E);
  double lQ = std::log(1.0 + 2.0 * Qmax / ELECTRON_MASS);
  double Delta = ALPHA_EM / (2 * PI) * (std::log(2.0 * gamma) - lQ / 3.0) * lQ * lQ;
  double delta = density_effect(sh, gamma);
  return 2 * PI * ELECTRON_RADIUS * ELECTRON_RADIUS * ELECTRON_MASS * AVOGADRO_NUMBER *
         m.ZoA / (beta2 * 1e-3) *
         (std::log(2.0 * ELECTRON_MASS * beta2 * gamma * gamma * Qmax / (m.I * m.I)) -
          2.0 * beta2 - delta + 0.25 * Qmax * Qmax / (E * E) + Delta);
}

// ------------------------------------------------------------ ionisation
// src/Materials.jl:513-528 (Salvat NIMB 316 (2013))
double electronic_dcs(double Z, double I, double m, double K, double q) {
  double P2 = K * (K + 2.0 * m), E = K + m;
  double Wmax = 2.0 * ELECTRON_MASS * P2 / (m * m + ELECTRON_MASS * (ELECTRON_MASS + 2.0 * E));
  if (q > Wmax) return 0.0;
  double Wmin = (13.6 / 19.2) * I;
  if (q <= Wmin) return 0.0;
  double E2 = E * E, beta2 = P2 / E2, a0 = 0.5 / E2, a1 = beta2 / Wmax;
  return 2 * PI * ELECTRON_MASS * ELECTRON_RADIUS * ELECTRON_RADIUS * Z *
         (a0 + 1.0 / q * (1.0 / q - a1)) / beta2;
}

// src/Materials.jl:536-570
double dcs_ionisation_integrate(double Z, double A, double I, double mass, double K,
                                double xlow, double xhigh, int mode) {
  double P2 = K * (K + 2.0 * mass), E = K + mass;
  double Wr = 2.0 * ELECTRON_MASS * P2 / (mass * mass + ELECTRON_MASS * (ELECTRON_MASS + 2.0 * E));
  double qlo = K * xlow, qhi = K * xhigh, Wmax = Wr;
  if (Wmax < qlo) return 0.0;
  if (Wmax > qhi) Wmax = qhi;
  double Wmin = (13.6 / 19.2) * I;
  if (qlo >= Wmin) Wmin = qlo;
  if (Wmax <= Wmin) return 0.0;
  double E2 = E * E, beta2 = P2 / E2, a0 = 0.5 / E2, a1 = beta2 / Wr, v;
  if (mode == 0)
    v = a0 * (Wmax - Wmin) - a1 * std::log(Wmax / Wmin) + 1.0 / Wmin - 1.0 / Wmax;
  else if (mode == 1)
    v = 0.5 * a0 * (Wmax * Wmax - Wmin * Wmin) - a1 * (Wmax - Wmin) + std::log(Wmax / Wmin);
  else
    v = a0 * (Wmax * Wmax * Wmax - Wmin * Wmin * Wmin) / 3.0 -
        0.5 * a1 * (Wmax * Wmax - Wmin * Wmin) + Wmax - Wmin;
  return 2 * PI * ELECTRON_MASS * ELECTRON_RADIUS * ELECTRON_RADIUS * Z * AVOGADRO_NUMBER /
         (A * 1e-3 * beta2) * v;
}

// ------------------------------------------------------------ radiative DCS
// src/Materials.jl:576-620: radiation logarithms (Z = 1..92, 0 = use 182.7)
double radiation_logarithm(double Z) {
  static const std::map<int, double> tab = {
      {1, 202.4}, {2, 151.9}, {3, 159.9}, {4, 172.3}, {5, 177.9}, {6, 178.3},
      {7, 176.6}, {8, 173.4}, {9, 170.0}, {10, 165.8}, {11, 165.8}, {12, 167.1},
      {13, 169.1}, {14, 170.8}, {15, 172.2}, {16, 173.4}, {17, 174.3}, {18, 174.8},
      {19, 175.1}, {20, 175.6}, {21, 176.2}, {22, 176.8}, {26, 175.8}, {29, 173.1},
      {32, 173.0}, {35, 173.5}, {42, 175.9}, {50, 177.4}, {53, 178.6}, {74, 177.6},
      {82, 178.0}, {92, 179.8}};
  auto it = tab.find(int(std::lround(Z)));
  return it == tab.end() ? 182.7 : it->second;
}

static const double SQRTE = 1.648721270700128;
static const double ME_MEV = 0.5109989461;
static const double RE_CM = 2.8179403227e-13;
static const double MMU_MEV = 105.6583745;

// src/Materials.jl:631-695 (Sandrock-Soedingrekso-Rhode bremsstrahlung)
double dcs_bremsstrahlung_ssr(double Z, double A, double m, double K, double q) {
  if (Z <= 0 || A <= 0 || m <= 0 || K <= 0 || q <= 0) return 0.0;
  double z13 = std::pow(Z, 1.0 / 3.0);
  if (q >= K + m * (1.0 - 0.75 * SQRTE * z13)) return 0.0;
  double energy = (K + m) * 1e3, v = q * 1e3 / energy, m_mev = m * 1e3;
  double Z13 = 1.0 / z13;
  double rl = radiation_logarithm(Z);
  double rl_inel = Z == 1.0 ? 446.0 : 1429.0;
  double Dn = 1.54 * std::pow(A, 0.27);
  double mu_qc = m_mev / (MMU_MEV * std::exp(1.0) / Dn);
  double rho = std::sqrt(1.0 + 4.0 * mu_qc * mu_qc);
  double log_rho = std::log((rho + 1.0) / (rho - 1.0));
  double delta1 = std::log(mu_qc) + 0.5 * rho * log_rho;
  double delta2 = std::log(mu_qc) + 0.25 * (3.0 * rho - rho * rho * rho) * log_rho +
                  2.0 * mu_qc * mu_qc;
  double delta = m_mev * m_mev * v / (2.0 * energy * (1.0 - v));
  double phi1 = std::log(rl * Z13 * (m_mev / ME_MEV) /
                         (1.0 + rl * Z13 * std::exp(0.5) * delta / ME_MEV));
  double phi2 = std::log(rl * Z13 * std::exp(-1.0 / 6.0) * (m_mev / ME_MEV) /
                         (1.0 + rl * Z13 * std::exp(1.0 / 3.0) * delta / ME_MEV));
  phi1 -= delta1 * (1.0 - 1.0 / Z);
  phi2 -= delta2 * (1.0 - 1.0 / Z);
  double sa1 = std::log(m_mev / delta / (m_mev * delta / (ME_MEV * ME_MEV) + SQRTE));
  double sa2 = std::log(1.0 + ME_MEV / (delta * rl_inel * Z13 * Z13 * SQRTE));
  double s_atomic = (4.0 / 3.0 * (1.0 - v) + v * v) * (sa1 - sa2);
  double s_rad;
  if (v < 0.0 || v > 1.0) {
    s_rad = 0.0;
  } else if (v < 0.02) {
    s_rad = -0.00349 + 148.84 * v + -987.531 * v * v;
  } else if (v < 0.1) {
    s_rad = 0.1642 + 132.573 * v + -585.361 * v * v + 1407.77 * v * v * v;
  } else if (v < 0.9) {
    double t = std::log(1.0 - v);
    s_rad = -2.8922 + -19.0156 * v + 57.698 * v * v;
    s_rad += -63.418 * v * std::log(v) + 14.1166 * t + 1.84206 * t * t;
  } else {
    double t = std::log(1.0 - v);
    s_rad = 2134.19 + 581.823 * v + -2708.85 * v * v;
    s_rad += 4767.05 * v * std::log(v) + 1.52918 * t + 0.361933 * t * t;
  }
  double res = ((2.0 - 2.0 * v + v * v) * phi1 - 2.0 / 3.0 * (1.0 - v) * phi2) +
               1.0 / Z * s_atomic + 0.25 * ALPHA_EM * phi1 * s_rad;
  if (res <= 0.0) return 0.0;
  double aux = 2.0 * (ME_MEV / m_mev) * RE_CM * Z;
  return aux * aux * (ALPHA_EM / q) * res * 1e-4;
}

// src/Materials.jl:701-800 (SSR pair production, double differential in rho)
static double pair_d2(double Z, double A, double mass, double K, double q, double rho_in) {
  double energy = (K + mass) * 1e3, v = q / (K + mass), m = mass * 1e3;
  double rl = radiation_logarithm(Z);
  double cpf = 4.0 / (3.0 * PI) * Z * (ALPHA_EM * RE_CM) * (ALPHA_EM * RE_CM);
  double Z13 = std::pow(Z, -1.0 / 3.0), dn = 1.54 * std::pow(A, 0.27);
  double rho = 1.0 - rho_in, rho2 = rho * rho;
  double g1 = Z == 1.0 ? 4.4e-5 : 1.95e-5, g2 = Z == 1.0 ? 4.8e-5 : 5.3e-5;
  double zeta1 = 0.073 * std::log(energy / m / (1.0 + g1 * std::pow(Z, 2.0 / 3.0) * energy / m)) - 0.26;
  double zeta2 = 0.058 * std::log(energy / m / (1.0 + g2 / Z13 * energy / m)) - 0.14;
  double zeta = (zeta1 > 0.0 && zeta2 > 0.0) ? zeta1 / zeta2 : 0.0;
  double beta = v * v / (2.0 * (1.0 - v));
  double xi = (m * v / (2.0 * ME_MEV)) * (m * v / (2.0 * ME_MEV)) * (1.0 - rho2) / (1.0 - v);
  double lxi = std::log(1.0 + 1.0 / xi);
  double Be = ((2.0 + rho2) * (1.0 + beta) + xi * (3.0 + rho2)) * lxi +
              (1.0 - rho2 - beta) / (1.0 + xi) - (3.0 + rho2);
  double Ce2 = ((1.0 - rho2) * (1.0 + beta) + xi * (3.0 - rho2)) * lxi +
               2.0 * (1.0 - beta - rho2) / (1.0 + xi) - (3.0 - rho2);
  double Ce1 = Be - Ce2;
  double De = ((2.0 + rho2) * (1.0 + beta) + xi * (3.0 + rho2)) * math_dilog(1.0 / (1.0 + xi)) -
              (2.0 + rho2) * xi * lxi - (xi + rho2 + beta) / (1.0 + xi);
  double den = energy * v * (1.0 - rho2);
  double Le1, Le2;
  if (De / Be > 0.0) {
    double t = De / Be, Xe = t < 100.0 ? std::exp(-t) : 0.0;
    Le1 = std::log(rl * Z13 * std::sqrt(1.0 + xi) /
                   (Xe + 2.0 * ME_MEV * std::exp(0.5) * rl * Z13 * (1.0 + xi) / den)) -
          t - 0.5 * std::log(Xe + (ME_MEV / m * dn) * (ME_MEV / m * dn) * (1.0 + xi));
    Le2 = std::log(rl * Z13 * std::exp(-1.0 / 6.0) * std::sqrt(1.0 + xi) /
                   (Xe + 2.0 * ME_MEV * std::exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den)) -
          t - 0.5 * std::log(Xe + (ME_MEV / m * dn) * (ME_MEV / m * dn) * std::exp(-1.0 / 3.0) * (1.0 + xi));
  } else {
    double t = De / Be, Xi = t > -100.0 ? std::exp(t) : 0.0;
    Le1 = std::log(rl * Z13 * std::sqrt(1.0 + xi) /
                   (1.0 + Xi * 2.0 * ME_MEV * std::exp(0.5) * rl * Z13 * (1.0 + xi) / den)) -
          0.5 * t - 0.5 * std::log(1.0 + Xi * (ME_MEV / m * dn) * (ME_MEV / m * dn) * (1.0 + xi));
    Le2 = std::log(rl * Z13 * std::exp(-1.0 / 6.0) * std::sqrt(1.0 + xi) /
                   (1.0 + Xi * 2.0 * ME_MEV * std::exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den)) -
          0.5 * t -
          0.5 * std::log(1.0 + Xi * (ME_MEV / m * dn) * (ME_MEV / m * dn) * std::exp(-1.0 / 3.0) * (1.0 + xi));
  }
  double de = cpf * (Z + zeta) * (1.0 - v) / v * (Ce1 * Le1 + Ce2 * Le2);
  if (de < 0.0) de = 0.0;
  double l1x = std::log(1.0 + xi);
  double Bm = ((1.0 + rho2) * (1.0 + 1.5 * beta) - 1.0 / xi * (1.0 + 2.0 * beta) * (1.0 - rho2)) * l1x +
              xi * (1.0 - rho2 - beta) / (1.0 + xi) + (1.0 + 2.0 * beta) * (1.0 - rho2);
  double Cm2 = ((1.0 - beta) * (1.0 - rho2) - xi * (1.0 + rho2)) * l1x / xi -
               2.0 * (1.0 - beta - rho2) / (1.0 + xi) + 1.0 - beta - (1.0 + beta) * rho2;
  double Cm1 = Bm - Cm2;
  double Dm = ((1.0 + rho2) * (1.0 + 1.5 * beta) - 1.0 / xi * (1.0 + 2.0 * beta) * (1.0 - rho2)) *
                  math_dilog(xi / (1.0 + xi)) +
              (1.0 + 1.5 * beta) * (1.0 - rho2) / xi * l1x +
              (1.0 - rho2 - 0.5 * beta * (1.0 + rho2) + (1.0 - rho2) / (2.0 * xi) * beta) * xi / (1.0 + xi);
  double Lm1, Lm2;
  if (Dm / Bm > 0.0) {
    double t = Dm / Bm, Xm = t < 100.0 ? std::exp(-t) : 0.0;
    Lm1 = std::log(m / ME_MEV * rl * Z13 / dn /
                   (Xm + 2.0 * ME_MEV * std::exp(0.5) * rl * Z13 * (1.0 + xi) / den)) - t;
    Lm2 = std::log(m / ME_MEV * rl * Z13 / dn /
                   (Xm + 2.0 * ME_MEV * std::exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den)) - t;
  } else {
    double t = Dm / Bm, Xv = t > -100.0 ? std::exp(t) : 0.0;
    Lm1 = std::log(m / ME_MEV * rl * Z13 / dn /
                   (1.0 + 2.0 * ME_MEV * std::exp(0.5) * rl * Z13 * (1.0 + xi) / den * Xv));
    Lm2 = std::log(m / ME_MEV * rl * Z13 / dn /
                   (1.0 + 2.0 * ME_MEV * std::exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den * Xv));
  }
  double dm = cpf * (Z + zeta) * (1.0 - v) / v * (ME_MEV / m) * (ME_MEV / m) * (Cm1 * Lm1 + Cm2 * Lm2);
  if (dm < 0.0) dm = 0.0;
  return (de + dm) * 0.1 / energy;
}

// src/Materials.jl:802-832
double dcs_pair_production_ssr(double Z, double A, double mass, double K, double q) {
  if (Z <= 0 || A <= 0 || mass <= 0 || K <= 0 || q <= 0) return 0.0;
  if (q <= 4.0 * ELECTRON_MASS) return 0.0;
  const double sqrte = 1.6487212707;
  double Z13 = std::pow(Z, 1.0 / 3.0);
  if (q >= K + mass * (1.0 - 0.75 * sqrte * Z13)) return 0.0;
  double gamma = 1.0 + K / mass;
  double x0 = 1.0 - 4.0 * ELECTRON_MASS / q;
  double x1 = 1.0 - 6.0 / (gamma * (gamma - q / mass));
  if (!(x0 > 0.0 && x1 > 0.0)) return 0.0;
  double rmax = std::sqrt(x0) * x1, ri = 1.0 - rmax;
  if (ri <= 0.0 || ri >= 1.0) return 0.0;
  double tmin = std::log(ri);
  const GQ& g = gq(12);
  double I = 0;
  for (int i = 0; i < 12; ++i) {
    double r = std::exp(g.x[i] * tmin);
    I -= pair_d2(Z, A, mass, K, q, r) * r * g.w[i] * tmin;
  }
  return I < 0.0 ? 0.0 : I;
}

// src/Materials.jl:838-926 (DRSS photonuclear with ALLM97 structure function)
static double f2p_allm97(double x, double Q2) {
  const double m02 = 0.31985, mP2 = 49.457, mR2 = 0.15052, Q02 = 0.52544, L2 = 0.06527;
  const double cP1 = 0.28067, cP2 = 0.22291, cP3 = 2.1979;
  const double aP1 = -0.0808, aP2 = -0.44812, aP3 = 1.1709;
  const double bP1 = 0.36292, bP2 = 1.8917, bP3 = 1.8439;
  const double cR1 = 0.80107, cR2 = 0.97307, cR3 = 3.4942;
  const double aR1 = 0.58400, aR2 = 0.37888, aR3 = 2.6063;
  const double bR1 = 0.01147, bR2 = 3.7582, bR3 = 0.49338;
  double M = 0.5 * (PROTON_MASS + NEUTRON_MASS), M2 = M * M;
  double W2 = M2 + Q2 * (1.0 / x - 1.0);
  double t = std::log(std::log((Q2 + Q02) / L2) / std::log(Q02 / L2));
  double xP = (Q2 + mP2) / (Q2 + mP2 + W2 - M2);
  double xR = (Q2 + mR2) / (Q2 + mR2 + W2 - M2);
  double cP = cP1 + (cP1 - cP2) * (1.0 / (1.0 + std::pow(t, cP3)) - 1.0);
  double aP = aP1 + (aP1 - aP2) * (1.0 / (1.0 + std::pow(t, aP3)) - 1.0);
  double bP = bP1 + bP2 * std::pow(t, bP3);
  double cR = cR1 + cR2 * std::pow(t, cR3);
  double aR = aR1 + aR2 * std::pow(t, aR3);
  double bR = bR1 + bR2 * std::pow(t, bR3);
  double F2P = cP * std::exp(aP * std::log(xP) + bP * std::log(1.0 - x));
  double F2R = cR * std::exp(aR * std::log(xR) + bR * std::log(1.0 - x));
  return Q2 / (Q2 + m02) * (F2P + F2R);
}
static double shadowing_drss(double Z, double A, double x) {
  if (Z == 1.0) return 1.0;
  if (x < 0.0014) return std::exp(-0.1 * std::log(A));
  if (x < 0.04) return std::exp((0.069 * std::log10(x) + 0.097) * std::log(A));
  return 1.0;
}
static double photo_d2(double Z, double A, double ml, double K, double q, double Q2) {
  double cf = 4 * PI * ALPHA_EM * ALPHA_EM * HBAR_C * HBAR_C;
  double M = 0.5 * (PROTON_MASS + NEUTRON_MASS), E = K + ml, y = q / E;
  double x = 0.5 * Q2 / (M * q);
  double F2p = f2p_allm97(x, Q2);
  double sh = shadowing_drss(Z, A, x);
  double F2A = F2p * sh * (Z + (A - Z) * (1.0 + x * (-1.85 + x * (2.45 + x * (-2.35 + x)))));
  double dds = (1.0 - y + 0.5 * (1.0 - 2.0 * ml * ml / Q2) * (y * y + Q2 / (E * E))) / (Q2 * Q2) -
               0.25 / (E * E * Q2);
  return cf * F2A * dds / q;
}
double dcs_photonuclear_drss(double Z, double A, double m, double K, double q) {
  if (Z <= 0 || A <= 0 || m <= 0 || K <= 0 || q <= 0) return 0.0;
  double M = 0.5 * (NEUTRON_MASS + PROTON_MASS), mpi = PION_MASS;
  double qmin = mpi + 0.5 * mpi * mpi / M, qmax = K + m - 0.5 * (M + m * m / M);
  if (q <= qmin || q >= qmax) return 0.0;
  double E = K + m, ml2 = m * m;
  double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
  double Q2max = 2.0 * M * (q - mpi) - mpi * mpi;
  if (Q2max < Q2min || Q2min < 0.0) return 0.0;
  const GQ& g = gq(9);
  double lmin = std::log(Q2min), dx = std::log(Q2max) - lmin, ds = 0;
  for (int i = 0; i < 9; ++i) {
    double Q2 = std::exp(lmin + dx * g.x[i]);
    double v = photo_d2(Z, A, m, K, q, Q2);
    if (v > 0.0) ds += v * (g.w[i] * dx * Q2);
  }
  return ds < 0.0 ? 0.0 : ds;
}

// src/Materials.jl:939-1007: energy moments of the raw DCS, 9-point GQ on
// (npoints+8)/9 equal log-q intervals.
double compute_dcs_integral(int proc, double Z, double A, double I, double mass, double K,
                            double xlow, double xhigh, int mode, int npoints) {
  if (xlow <= 0.0) xlow = 1e-6;
  if (proc == IONI) return dcs_ionisation_integrate(Z, A, I, mass, K, xlow, xhigh, mode);
  double M = 0.5 * (NEUTRON_MASS + PROTON_MASS), mpi = PION_MASS, qmin, qmax;
  if (proc == PHOTO) {
    qmin = mpi + 0.5 * mpi * mpi / M;
    qmax = K + mass - 0.5 * (M + mass * mass / M);
  } else {
    double Z13 = std::pow(Z, 1.0 / 3.0);
    qmax = K + mass * (1.0 - 0.75 * 1.648721271 * Z13);
    qmin = proc == PAIR ? 4.0 * ELECTRON_MASS : 0.0;
  }
  double qlo = std::max(xlow * K, qmin), qhi = std::min(xhigh * K, qmax);
  if (qlo >= qhi) return 0.0;
  int nint = (npoints + 8) / 9;
  const GQ& g = gq(9);
  double lo = std::log(qlo), hi = std::log(qhi), s = 0;
  for (int k = 0; k < nint; ++k) {
    double a = lo + k * (hi - lo) / nint, b = lo + (k + 1) * (hi - lo) / nint, dx = b - a;
    for (int j = 0; j < 9; ++j) {
      double x = std::exp(a + dx * g.x[j]), w = g.w[j] * dx * x, v;
      if (proc == BREMS) v = dcs_bremsstrahlung_ssr(Z, A, mass, K, x);
      else if (proc == PAIR) v = dcs_pair_production_ssr(Z, A, mass, K, x);
      else v = dcs_photonuclear_drss(Z, A, mass, K, x);
      if (mode >= 1) v *= x;
      if (mode >= 2) v *= x;
      s += v * w;
    }
  }
  return s * AVOGADRO_NUMBER / (A * 1e-3);
}

}  // namespace orc

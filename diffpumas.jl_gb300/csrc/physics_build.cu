// physics_build.cu -- host-side construction of the muon physics tables,
// the product counterpart of create_physics(MUON): src/Physics.jl:280-408
// (create_material_table_empirical, no PUMAS dE/dx files), :146-273
// (create_material_table_from_dedx) with src/DEDXLoader.jl:49-190
// (load_dedx_file), :534-599 (create_physics), src/Materials.jl:360-507
// (atomic shells, Fano density effect, electronic stopping) and :939-1007
// (DCS energy moments).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <thread>
#include <vector>

#include "dcs.cuh"
#include "internal.h"
#include "physics_data.inc"

namespace dp {
namespace {

struct Shell {
  double f, E;
};

void add_shells(int Z, double w, std::vector<Shell>& out) {
  int iZ = std::min(std::max(Z, 1), 100);
  for (int s = DPDATA_SHELL_INDEX[iZ - 1]; s < DPDATA_SHELL_INDEX[iZ]; ++s)
    out.push_back({w * double(DPDATA_SHELL_OCCUPANCY[s]), double(DPDATA_SHELL_ENERGY_EV[s])});
}

// src/Materials.jl:404-431 (atomic_shell_create + atomic_shell_normalise!)
std::vector<Shell> material_shells(const HostMaterial& m) {
  std::vector<Shell> sh;
  for (const auto& e : m.elements) {
    double w = e.fraction / e.A;
    if (e.Z == 11.0 && e.A == 22.0) {  // standard-rock pseudo element: C + 3 O + Ca
      double ws = w * 11.0 / 50.0;
      add_shells(6, ws, sh);
      add_shells(8, 3.0 * ws, sh);
      add_shells(20, ws, sh);
    } else {
      add_shells(int(std::lround(e.Z)), w, sh);
    }
  }
  double ftot = 0.0, lnI = 0.0;
  for (const auto& s : sh) {
    ftot += s.f;
    lnI += s.f * std::log(s.E);
  }
  lnI /= ftot;
  double wp = 28.816 * std::sqrt(m.ZoA * m.density * 1e-3);
  double r = (m.I * 1e9 / std::exp(lnI)) / wp;
  for (auto& s : sh) {
    s.f /= ftot;
    s.E *= r;
  }
  return sh;
}

// src/Materials.jl:437-469: Fano density effect by bisection on l^2.
double density_effect(const std::vector<Shell>& sh, double gamma) {
  double y = 1.0 / (gamma * gamma), ymax = 0.0;
  for (const auto& s : sh) ymax += s.f / (s.E * s.E);
  if (ymax <= y) return 0.0;
  double lo = 0.0, hi = 1.0 / y, l2 = 0.0;
  for (int it = 0; it < 200; ++it) {
    l2 = 0.5 * (lo + hi);
    double yi = 0.0;
    for (const auto& s : sh) yi += s.f / (s.E * s.E + l2);
    if (std::fabs(yi - y) <= kEps64 || (hi - lo) <= kEps64) break;
    if (yi > y) lo = l2; else hi = l2;
  }
  double d = -l2 * y;
  for (const auto& s : sh) d += s.f * std::log(1.0 + l2 / (s.E * s.E));
  return d;
}

// src/Materials.jl:488-507
double electronic_stopping(const HostMaterial& m, const std::vector<Shell>& sh, double mass,
                           double K) {
  double E = K + mass, P2 = K * (K + 2.0 * mass), b2 = P2 / (E * E), g = E / mass;
  double r = kElectronMass / mass;
  double Qmax = 2.0 * r * P2 / (mass * (1.0 + r * r) + 2.0 * r * E);
  double lQ = std::log(1.0 + 2.0 * Qmax / kElectronMass);
  double Delta = kAlpha / (2.0 * kPi) * (std::log(2.0 * g) - lQ / 3.0) * lQ * lQ;
  return 2.0 * kPi * kElectronRadius * kElectronRadius * kElectronMass * kAvogadro * m.ZoA /
         (b2 * 1e-3) *
         (std::log(2.0 * kElectronMass * b2 * g * g * Qmax / (m.I * m.I)) - 2.0 * b2 -
          density_effect(sh, g) + 0.25 * Qmax * Qmax / (E * E) + Delta);
}

// src/Materials.jl:536-570: closed-form moments of the ionisation DCS.
double ionisation_moment(double Z, double A, double I, double mass, double K, double xlo,
                         double xhi, int mode) {
  double P2 = K * (K + 2.0 * mass), E = K + mass;
  double Wr = 2.0 * kElectronMass * P2 / (mass * mass + kElectronMass * (kElectronMass + 2.0 * E));
  double qlo = K * xlo, qhi = K * xhi, Wmax = Wr;
  if (Wmax < qlo) return 0.0;
  if (Wmax > qhi) Wmax = qhi;
  double Wmin = std::max((13.6 / 19.2) * I, qlo);
  if (Wmax <= Wmin) return 0.0;
  double E2 = E * E, b2 = P2 / E2, a0 = 0.5 / E2, a1 = b2 / Wr, v;
  if (mode == 0)
    v = a0 * (Wmax - Wmin) - a1 * std::log(Wmax / Wmin) + 1.0 / Wmin - 1.0 / Wmax;
  else if (mode == 1)
    v = 0.5 * a0 * (Wmax * Wmax - Wmin * Wmin) - a1 * (Wmax - Wmin) + std::log(Wmax / Wmin);
  else
    v = a0 * (Wmax * Wmax * Wmax - Wmin * Wmin * Wmin) / 3.0 - 0.5 * a1 * (Wmax * Wmax - Wmin * Wmin) +
        Wmax - Wmin;
  return 2.0 * kPi * kElectronMass * kElectronRadius * kElectronRadius * Z * kAvogadro /
         (A * 1e-3 * b2) * v;
}

enum { P_BREMS = 0, P_PAIR = 1, P_PHOTO = 2, P_IONI = 3 };

// src/Materials.jl:939-1007: energy moment `mode` of process `proc` between
// xlo*K and xhi*K, 9-point Gauss-Legendre on 20 equal log-q intervals.
double dcs_moment(int proc, double Z, double A, double I, double mass, double K, double xlo,
                  double xhi, int mode) {
  if (xlo <= 0.0) xlo = 1e-6;
  if (proc == P_IONI) return ionisation_moment(Z, A, I, mass, K, xlo, xhi, mode);
  double M = 0.5 * (kNeutronMass + kProtonMass), qmin, qmax;
  if (proc == P_PHOTO) {
    qmin = kPionMass + 0.5 * kPionMass * kPionMass / M;
    qmax = K + mass - 0.5 * (M + mass * mass / M);
  } else {
    qmax = K + mass * (1.0 - 0.75 * 1.648721271 * std::pow(Z, 1.0 / 3.0));
    qmin = proc == P_PAIR ? 4.0 * kElectronMass : 0.0;
  }
  double qlo = std::max(xlo * K, qmin), qhi = std::min(xhi * K, qmax);
  if (qlo >= qhi) return 0.0;
  const int nint = 20;
  double a0 = std::log(qlo), a1 = std::log(qhi), s = 0.0;
  for (int k = 0; k < nint; ++k) {
    double a = a0 + k * (a1 - a0) / nint, b = a0 + (k + 1) * (a1 - a0) / nint, h = b - a;
    for (int j = 0; j < 9; ++j) {
      double q = std::exp(a + h * gl9(j, false)), wq = gl9(j, true) * h * q;
      double v = proc == P_BREMS ? dcs_brems(Z, A, mass, K, q)
                 : proc == P_PAIR ? dcs_pair(Z, A, mass, K, q)
                                  : dcs_photo(Z, A, mass, K, q);
      if (mode >= 1) v *= q;
      if (mode >= 2) v *= q;
      s += v * wq;
    }
  }
  return s * kAvogadro / (A * 1e-3);
}

// ------------------------------------------------------------ Coulomb tables
// src/Coulomb.jl: Salvat's screened Coulomb DCS (three exponentials plus a
// nuclear-size term), reduced to simple poles, with the KTV Born correction;
// the first transport path adds the electronic transverse transport and the
// radiative soft-scattering integrals below the cutoff.

// Nuclear radius by the reference's C-index rule (src/Coulomb.jl:166-181):
// hydrogen with A >= 1.5 uses the first entry, the standard-rock pseudo
// element (Z 11, A 22) the last one.
double nuclear_radius(double Z, double A) {
  const int nN = 120;
  int iN = int(Z);
  if (iN >= nN - 1) iN = nN - 2;
  else if (iN == 1 && A >= 1.5) iN = 0;
  else if (iN == 11 && A == 22.0) iN = nN - 1;
  return DPDATA_NUCLEAR_RADII_FM[iN] * 1e-15;
}

// Centre-of-mass frame of the muon-nucleus collision (src/Coulomb.jl:192-206).
void cm_frame(double Z, double A, double mass, double K, double* K0, double* gCM, double* tau) {
  double Ma = Z * kProtonMass + (A - Z) * kNeutronMass;
  double s12i = 1.0 / std::sqrt((mass + Ma) * (mass + Ma) + 2.0 * Ma * K);
  *gCM = (K + mass + Ma) * s12i;
  double k0 = (K * Ma + mass * (mass + Ma)) * s12i - mass;
  *K0 = k0 < 1e-9 ? 1e-9 : k0;
  double et = K + mass + Ma, b2 = K * (K + 2.0 * mass) / (et * et), rm = mass / Ma;
  *tau = std::sqrt(rm * rm * (1.0 - b2) + b2);
}

// Inverse of the DCS normalisation per unit mass (src/Coulomb.jl:211-217).
double cm_normalisation(double Z, double A, double mass, double K, double K0) {
  double p2 = K * (K + 2.0 * mass), p02 = K0 * (K0 + 2.0 * mass);
  double d = kAlpha * Z * kHbarC * (K + mass);
  return A * 1e-3 * p2 * p02 / (d * d * kPi * kAvogadro);
}

// Screening amplitudes and parameters; the last parameter is the nuclear
// term (src/Coulomb.jl:224-289).
struct Screening {
  int n = 0;
  double amp[4] = {0, 0, 0, 0}, par[5] = {0, 0, 0, 0, 0};
};
Screening screening(double Z, double A, double mass, double K, double K0) {
  double aZE = kAlpha * Z * (K + mass), z2 = aZE * aZE / (K * (K + 2.0 * mass)), f;
  if (z2 < 1.0) {
    f = z2 * (1.0 / (1.0 + z2) + 0.20205690315959424 - 0.03692775514336999 * z2 +
              0.008349277381922926 * z2 * z2);
  } else {
    double r2i = 1.0 / (1.0 + z2), phi = -std::atan(std::sqrt(z2));
    f = -0.5 * std::log(r2i) + 0.5 * (1.0 - r2i) + (1.0 - std::cos(2 * phi) * r2i) / 12.0 -
        (1.0 - std::cos(4 * phi) * r2i * r2i) / 120.0 +
        (1.0 - std::cos(6 * phi) * r2i * r2i * r2i) / 252.0;
  }
  double d = 0.25 * kHbarC * kHbarC / (K0 * (K0 + 2.0 * mass)) * std::exp(2.0 * f);
  int iZ = std::min(std::max(int(Z) - 1, 0), 102);
  Screening s;
  int n;
  if (DPDATA_SALVAT_EXPONENT2[iZ] == 1.0) {
    n = iZ == 0 ? 1 : 2;
    s.amp[0] = iZ == 0 ? 1.0 : DPDATA_SALVAT_PREFACTOR0[iZ];
    if (n == 2) s.amp[1] = 1.0 - s.amp[0];
  } else {
    n = 3;
    s.amp[0] = DPDATA_SALVAT_PREFACTOR0[iZ];
    s.amp[1] = DPDATA_SALVAT_PREFACTOR1[iZ];
    s.amp[2] = 1.0 - (s.amp[0] + s.amp[1]);
  }
  const double* ex[3] = {DPDATA_SALVAT_EXPONENT0, DPDATA_SALVAT_EXPONENT1, DPDATA_SALVAT_EXPONENT2};
  for (int i = 0; i < n; ++i) {
    double a = ex[i][iZ] / kBohrRadius;
    s.par[i] = d * a * a;
  }
  double RN = nuclear_radius(Z, A);
  s.par[n] = 12.0 * d / (RN * RN);
  s.n = n + 1;
  return s;
}

// Partial fractions of the screened DCS times the nuclear form factor
// (src/Coulomb.jl:292-348).
struct Poles {
  double a[3] = {0, 0, 0}, b[3] = {0, 0, 0}, c[4] = {0, 0, 0, 0};
};
Poles poles(const Screening& s) {
  Poles P;
  const int n = s.n - 1;
  for (int i = 0; i < n; ++i) {
    P.b[i] = s.amp[i] * s.amp[i];
    for (int j = i + 1; j < n; ++j) {
      double d = 2.0 * s.amp[i] * s.amp[j] / (s.par[j] - s.par[i]);
      P.a[i] += d;
      P.a[j] -= d;
    }
  }
  const double N = s.par[n];
  double Sa[4] = {0, 0, 0, 0}, Sb[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    double x = 1.0 - s.par[i] / N, r = x;
    for (int j = 0; j < 4; ++j) {
      Sa[j] += P.a[i] / r;
      r *= x;
      Sb[j] += P.b[i] / r;
    }
  }
  double t = 1.0;
  for (int i = 0; i < 4; ++i) {
    P.c[i] = ((4 - i) * Sb[3 - i] / N - Sa[3 - i]) * t;
    t *= N;
  }
  for (int i = 0; i < n; ++i) {
    double dd = 1.0 - s.par[i] / N, d4 = dd * dd * dd * dd;
    P.a[i] = (P.a[i] - 4.0 * P.b[i] / (N - s.par[i])) / d4;
    P.b[i] /= d4;
  }
  return P;
}

// Zeroth and (twice the) first transport coefficients of the cross section
// restricted to deflections below mu, spin factor S (src/Coulomb.jl:350-406).
void transport_coefs(double mu, double S, const Screening& s, const Poles& P, double* c0,
                     double* c1x2) {
  const int n = s.n - 1;
  double t0 = 0, t1 = 0;
  for (int i = 0; i < n; ++i) {
    double al = s.par[i], r = mu / (mu + al), L = std::log(1.0 + mu / al);
    double I0 = r / al, J0 = L, I1 = L - r, J1 = -al * L, I2 = mu + al * (r - 2.0 * L);
    double J2 = al * (al * L - mu);
    t0 += P.a[i] * (J0 - S * J1) + P.b[i] * (I0 - S * I1);
    t1 += P.a[i] * (J1 - S * J2) + P.b[i] * (I1 - S * I2);
  }
  const double N = s.par[n], r = mu / (mu + N), L = std::log(1.0 + mu / N);
  double I0 = r / N, J0 = L, I1 = L - r, J1 = -N * L, I2 = mu + N * (r - 2.0 * L),
         J2 = N * (N * L - mu);
  double rn = 1.0 / (1.0 + mu / N);
  double K0 = (1.0 - rn) * (1.0 + rn) / (2.0 * N * N);
  double L0 = (1.0 - rn) * ((1.0 + rn) * (1.0 + rn) - rn) / (3.0 * N * N * N);
  double K1 = I0 - N * K0, L1 = K0 - N * L0, K2 = I1 - N * K1, L2 = K1 - N * L1;
  t0 += P.c[0] * (J0 - S * J1) + P.c[1] * (I0 - S * I1) + P.c[2] * (K0 - S * K1) +
        P.c[3] * (L0 - S * L1);
  t1 += P.c[0] * (J1 - S * J2) + P.c[1] * (I1 - S * I2) + P.c[2] * (K1 - S * K2) +
        P.c[3] * (L1 - S * L2);
  *c0 = t0;
  *c1x2 = 2.0 * t1;
}

// Cross section of deflections above mu (src/Coulomb.jl:409-417).
double hard_cs(double mu, double S, const Screening& s, const Poles& P) {
  if (mu >= 1.0 || mu >= 1e6 * s.par[s.n - 1]) return 0.0;
  double f0, f1, m0, m1;
  transport_coefs(1.0, S, s, P, &f0, &f1);
  transport_coefs(mu, S, s, P, &m0, &m1);
  return m0 > f0 ? 0.0 : f0 - m0;
}

// Ridder's root bracketing (src/Coulomb.jl:428-471).
template <class F>
double ridder(F f, double xa, double xb, double fa, double fb, double xtol, double rtol,
              int maxiter) {
  if (fa * fb > 0) return 0.0;
  if (fa == 0) return xa;
  if (fb == 0) return xb;
  double tol = xtol + rtol * std::min(std::fabs(xa), std::fabs(xb)), xn = 0.0;
  for (int it = 0; it < maxiter; ++it) {
    double dm = 0.5 * (xb - xa), xm = xa + dm, fm = f(xm);
    double dn = (fb > fa ? 1.0 : -1.0) * dm * fm / std::sqrt(fm * fm - fa * fb);
    double sg = dn > 0.0 ? 1.0 : -1.0, step = std::fabs(dm) - 0.5 * tol;
    if (std::fabs(dn) < step) step = std::fabs(dn);
    xn = xm - sg * step;
    double fn = f(xn);
    if (fn * fm < 0.0) {
      xa = xn;
      fa = fn;
      xb = xm;
      fb = fm;
    } else if (fn * fa < 0.0) {
      xb = xn;
      fb = fn;
    } else {
      xa = xn;
      fa = fn;
    }
    if (fn == 0.0 || std::fabs(xb - xa) < tol) return xn;
  }
  return xn;
}

// Electronic transverse transport cross section (src/Coulomb.jl:493-510).
double electronic_transport(double ZoA, double I, double aS, double mass, double K, double nu) {
  double p2 = K * (K + 2.0 * mass), E = K + mass;
  double Wr = 2.0 * kElectronMass * p2 / (mass * mass + kElectronMass * (kElectronMass + 2.0 * E));
  double Wmax = std::min(nu, Wr), b2 = p2 / (E * E);
  double J = std::log(aS * Wmax / I) - b2 * Wmax / Wr + 0.25 * Wmax * Wmax / (E * E) + 1.0 / aS;
  double g = E / mass, lQ = std::log(1.0 + 2.0 * Wr / kElectronMass);
  double Delta = kAlpha / (2 * kPi) * (std::log(2.0 * g) - lQ / 3.0) * lQ * lQ;
  return 2 * kPi * kElectronRadius * kElectronRadius * kElectronMass * kElectronMass * kAvogadro *
         ZoA / (b2 * 1e-3 * p2) * (J + Delta);
}

// Gauss-Legendre rule on [0, 1] by Newton iteration on P_n.
struct GaussLegendre {
  double x[20], w[20];
  explicit GaussLegendre(int n) {
    for (int i = 0; i < n; ++i) {
      double z = std::cos(kPi * (i + 0.75) / (n + 0.5)), pp = 0;
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
      x[i] = 0.5 * (1.0 - z);
      w[i] = 1.0 / ((1.0 - z * z) * pp * pp);
    }
  }
};

// Angular transport integral of a radiative DCS over log q (src/Coulomb.jl:564-593).
template <class D>
double radiative_transport(D dcs, double Z, double A, double mass, double K, double qmin,
                           double qmax) {
  if (qmin >= qmax || qmin <= 0.0) return 0.0;
  static const GaussLegendre g(20);
  double p2 = K * (K + 2.0 * mass), lo = std::log(qmin), hi = std::log(qmax), r = 0.0;
  for (int i = 0; i < 20; ++i) {
    double q = std::exp(lo + (hi - lo) * g.x[i]), v = dcs(Z, A, mass, K, q);
    if (v > 0.0) r += v * (q * q / p2) * q * (g.w[i] * (hi - lo));
  }
  return r;
}

// Soft radiative scattering below the cutoff (src/Coulomb.jl:595-635).
double radiative_soft(double Z, double A, double mass, double K, double cutoff) {
  double qmaxp = K + mass * (1.0 - 0.75 * 1.6487212707 * std::pow(Z, 1.0 / 3.0));
  double qb = std::min(cutoff * K, qmaxp);
  double r = radiative_transport([](double z, double a, double m, double k, double q) {
    return dcs_brems(z, a, m, k, q); }, Z, A, mass, K, 1e-3 * qb, qb);
  r += radiative_transport([](double z, double a, double m, double k, double q) {
    return dcs_pair(z, a, m, k, q); }, Z, A, mass, K, std::max(4.0 * kElectronMass, 1e-3 * qb), qb);
  double qp = cutoff * K;
  r += radiative_transport([](double z, double a, double m, double k, double q) {
    return dcs_photo(z, a, m, k, q); }, Z, A, mass, K, std::max(0.0, 1e-3 * qp), qp);
  return r;
}

// compute_coulomb_tables! (src/Coulomb.jl:688-826) at one energy node:
// first transport path lb1, elastic path x p^2 lbe, screening cutoff mu0.
void coulomb_node(const HostMaterial& m, double mass, double elastic_ratio, double cutoff,
                  double aS, double K, double range, double* lb1, double* lbe, double* mu0_out) {
  if (K <= 0.0) {
    *lb1 = *lbe = *mu0_out = 0.0;
    return;
  }
  const size_t ne = m.elements.size();
  std::vector<Screening> sc(ne);
  std::vector<Poles> po(ne);
  std::vector<double> fs(ne), nf(ne), d2(ne);
  double cs_m = 0, cs1_m = 0, A_min = 1e300, cs_A = 0;
  for (size_t k = 0; k < ne; ++k) {
    const HostElement& el = m.elements[k];
    double K0, gCM, tau;
    cm_frame(el.Z, el.A, mass, K, &K0, &gCM, &tau);
    double e = K + mass;
    fs[k] = K * (e + mass) / (e * e);
    sc[k] = screening(el.Z, el.A, mass, K, K0);
    po[k] = poles(sc[k]);
    double G0, G1;
    transport_coefs(1.0, fs[k], sc[k], po[k], &G0, &G1);
    nf[k] = el.fraction / cm_normalisation(el.Z, el.A, mass, K, K0);
    cs_m += nf[k] * G0;
    double d = 1.0 / (gCM * (1.0 + tau));
    d2[k] = d * d;
    cs1_m += nf[k] * G1 * d2[k];
    for (int j = 0; j < sc[k].n - 1; ++j) A_min = std::min(A_min, sc[k].par[j]);
    cs_A += nf[k];
  }
  cs_A /= A_min * (A_min + 1.0);
  const double path_max = 1e9, max_mu0 = 0.5 * (1.0 - std::cos(kPi / 180.0));
  double cs_h = std::max(cs1_m, range > 0.0 ? 1.0 / range : 0.0) / elastic_ratio;
  if (cs_h < 1.0 / path_max) cs_h = 1.0 / path_max;
  double mu0, lb_h;
  if (cs_h < cs_m) {
    double zeta = cs_h / cs_A;
    double mu_max = std::min(A_min * (1.0 - zeta) / (A_min + zeta), max_mu0);
    auto obj = [&](double mu) {
      double t = 0;
      for (size_t k = 0; k < ne; ++k) t += nf[k] * hard_cs(mu, fs[k], sc[k], po[k]);
      return t - cs_h;
    };
    mu0 = ridder(obj, 0.0, mu_max, cs_m - cs_h, obj(mu_max), 1e-6 * mu_max, 1e-6, 100);
    if (mu0 > max_mu0) mu0 = max_mu0;
    cs_h += obj(mu0);
    lb_h = cs_h <= 1.0 / path_max ? path_max : 1.0 / cs_h;
  } else {
    mu0 = 0.0;
    lb_h = 1.0 / cs_m;
  }
  *mu0_out = mu0;
  *lbe = lb_h * K * (K + 2.0 * mass);
  double inv = 0;
  for (size_t k = 0; k < ne; ++k) {
    double G0, G1;
    transport_coefs(mu0, fs[k], sc[k], po[k], &G0, &G1);
    inv += nf[k] * d2[k] * G1;
  }
  double rad = 0;
  for (size_t k = 0; k < ne; ++k)
    rad += radiative_soft(m.elements[k].Z, m.elements[k].A, mass, K, cutoff) * m.elements[k].fraction;
  double tot = inv + rad + electronic_transport(m.ZoA, m.I, aS, mass, K, cutoff * K);
  *lb1 = tot > 0.0 ? 1.0 / tot : 0.0;
}

template <class F>
void parallel_for(int n, F f) {
  unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  std::vector<std::thread> th;
  std::atomic<int> next{0};
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&] {
      for (int i = next++; i < n; i = next++) f(i);
    });
  for (auto& x : th) x.join();
}

// Coulomb scattering tables (src/Physics.jl:386-397, :234-256 from the
// CSDA range and m.ZoA) and the per-node kinematic columns (spin factor,
// magnetic rotation, elastic cutoff angle).
void coulomb_and_kinematics(const HostMaterial& m, const dp_settings& st, int n, double* cols) {
  auto C = [&](int c) { return cols + size_t(c) * n; };
  const double mass = st.mass, cut = st.cutoff;
  const double *E = C(DP_COL_E), *R = C(DP_COL_CSDA_R);
  const double aS = m.I * 1e9 / (28.816 * std::sqrt(m.ZoA * m.density * 1e-3));
  parallel_for(n, [&](int i) {
    coulomb_node(m, mass, st.elastic_ratio, cut, aS, E[i], R[i], C(DP_COL_LB1) + i,
                 C(DP_COL_LBE) + i, C(DP_COL_MU0) + i);
  });
  for (int i = 0; i < n; ++i) {
    double K = E[i], g = 1.0 + K / mass, b = std::sqrt(1.0 - 1.0 / (g * g));
    double p = std::sqrt(K * (K + 2 * mass)), e = K + mass;
    C(DP_COL_FSPIN)[i] = K * (e + mass) / (e * e);
    C(DP_COL_MAGROT)[i] = kLarmor / (b * p);
    double mu0 = C(DP_COL_MU0)[i];
    C(DP_COL_ECUT)[i] = mu0 < 1e-8 ? 2.0 * std::sqrt(std::max(mu0, 0.0))
                                   : std::acos(std::max(1.0 - 2.0 * mu0, -1.0));
  }
}

}  // namespace

// src/Physics.jl:280-408.  Columns per DP_COL_*, the Coulomb scattering
// columns (LB1, LBE, MU0, ECUT) included.
void build_empirical_table(const HostMaterial& m, const dp_settings& st, int n, double Kmin,
                           double Kmax, double* cols /* DP_NCOL x n */) {
  auto C = [&](int c) { return cols + size_t(c) * n; };
  for (int c = 0; c < DP_NCOL; ++c) std::fill(C(c), C(c) + n, 0.0);
  double* E = C(DP_COL_E);
  for (int i = 0; i < n; ++i) {
    E[i] = Kmin * std::pow(Kmax / Kmin, double(i) / double(n - 1));
    C(DP_COL_LOGE)[i] = std::log(E[i]);
  }
  std::vector<Shell> sh = material_shells(m);
  const double mass = st.mass, cut = st.cutoff;
  parallel_for(n, [&](int i) {
    double K = E[i], br = 0, pa = 0, ph = 0, hard = 0, cs = 0, sg = 0;
    if (K >= 1e-6) {
      for (const auto& e : m.elements) {
        double f = e.fraction;
        br += f * dcs_moment(P_BREMS, e.Z, e.A, e.I, mass, K, 1e-6, 1.0, 1);
        pa += f * dcs_moment(P_PAIR, e.Z, e.A, e.I, mass, K, 1e-6, 1.0, 1);
        ph += f * dcs_moment(P_PHOTO, e.Z, e.A, e.I, mass, K, 1e-6, 1.0, 1);
        for (int p = 0; p < 4; ++p) {
          hard += f * dcs_moment(p, e.Z, e.A, e.I, mass, K, cut, 1.0, 1);
          cs += f * dcs_moment(p, e.Z, e.A, e.I, mass, K, cut, 1.0, 0);
        }
        sg += f * dcs_moment(P_IONI, e.Z, e.A, e.I, mass, K, 0.0, cut, 2);
      }
    }
    double el = electronic_stopping(m, sh, mass, K);
    C(DP_COL_ION)[i] = el;
    C(DP_COL_BREMS)[i] = br;
    C(DP_COL_PAIR)[i] = pa;
    C(DP_COL_PHOTO)[i] = ph;
    C(DP_COL_CSDA_S)[i] = el + br + pa + ph;
    C(DP_COL_MIXED_S)[i] = std::max(C(DP_COL_CSDA_S)[i] - hard, 1e-20);
    C(DP_COL_STRAG)[i] = sg;
    C(DP_COL_XS)[i] = cs;
  });
  // Trapezoid ranges and proper time (src/Physics.jl:364-388)
  double *S = C(DP_COL_CSDA_S), *Sm = C(DP_COL_MIXED_S), *R = C(DP_COL_CSDA_R),
         *Rm = C(DP_COL_MIXED_R), *T = C(DP_COL_CSDA_T);
  R[0] = E[0] / S[0];
  Rm[0] = E[0] / Sm[0];
  T[0] = 0.0;
  for (int i = 1; i < n; ++i) {
    double dK = E[i] - E[i - 1];
    R[i] = R[i - 1] + dK / ((S[i] + S[i - 1]) / 2);
    Rm[i] = Rm[i - 1] + dK / ((Sm[i] + Sm[i - 1]) / 2);
    double g = 1.0 + E[i] / mass, gp = 1.0 + E[i - 1] / mass;
    double b = std::sqrt(1.0 - 1.0 / (g * g)), bp = std::sqrt(1.0 - 1.0 / (gp * gp));
    T[i] = T[i - 1] + dK / (((S[i] + S[i - 1]) / 2) * ((b + bp) / 2) * ((g + gp) / 2));
  }
  coulomb_and_kinematics(m, st, n, cols);
}

// load_dedx_file (src/DEDXLoader.jl:49-190): the header up to the units line
// (<Z/A>), then every line of at least 11 numbers: T [MeV], p, ionisation,
// bremsstrahlung, pair, photonuclear, radiative, dE/dx [MeV cm^2/g], CSDA
// range [g/cm^2], delta, beta.  Lines that do not parse are skipped.
bool load_dedx_table(const char* path, DedxTable* t, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = std::string("DEDX file not found: ") + path;
    return false;
  }
  *t = DedxTable{};
  std::string line;
  bool data = false;
  while (std::getline(f, line)) {
    if (!data) {
      const size_t z = line.find("<Z/A>");
      if (z != std::string::npos) {
        const size_t eq = line.find("= ", z);
        if (eq != std::string::npos) {
          const char* s = line.c_str() + eq + 2;
          char* end = nullptr;
          const double v = std::strtod(s, &end);
          if (end != s && (std::isdigit(static_cast<unsigned char>(*s)) || *s == '.')) t->ZoA = v;
        }
      }
      if (line.find("[MeV]") != std::string::npos && line.find("[MeV/c]") != std::string::npos)
        data = true;
      continue;
    }
    std::istringstream is(line);
    std::string tok;
    double v[11];
    int k = 0;
    bool ok = true;
    while (k < 11 && is >> tok) {
      char* end = nullptr;
      v[k] = std::strtod(tok.c_str(), &end);
      if (end == tok.c_str() || *end != '\0') {
        ok = false;
        break;
      }
      ++k;
    }
    if (!ok || k < 11 || line.find_first_not_of(" \t") == std::string::npos) continue;
    const double conv_dedx = 1e-4, conv_range = 10.0;  // MeV cm^2/g, g/cm^2 -> kg/m^2
    t->K.push_back(v[0] * 1e-3);
    t->ion.push_back(v[2] * conv_dedx);
    t->brems.push_back(v[3] * conv_dedx);
    t->pair.push_back(v[4] * conv_dedx);
    t->photo.push_back(v[5] * conv_dedx);
    t->S.push_back(v[7] * conv_dedx);
    t->R.push_back(v[8] * conv_range);
  }
  if (!data) {
    *err = std::string("Could not find data section in DEDX file ") + path;
    return false;
  }
  if (t->K.size() < 2) {
    *err = std::string("no table rows in DEDX file ") + path;
    return false;
  }
  return true;
}

// src/Physics.jl:146-273.  Energies, CSDA stopping power and range and the
// four loss components come from the file; the proper time and restricted
// range are trapezoids; the hard loss, straggling and hard cross section
// (K >= 1e-3 GeV) are per-element DCS moments; the Coulomb columns use the
// file's <Z/A>.
void build_dedx_table(const HostMaterial& m, const DedxTable& t, const dp_settings& st,
                      double* cols) {
  const int n = int(t.K.size());
  auto C = [&](int c) { return cols + size_t(c) * n; };
  for (int c = 0; c < DP_NCOL; ++c) std::fill(C(c), C(c) + n, 0.0);
  const double mass = st.mass, cut = st.cutoff;
  double* E = C(DP_COL_E);
  for (int i = 0; i < n; ++i) {
    E[i] = t.K[i];
    C(DP_COL_LOGE)[i] = std::log(E[i]);
    C(DP_COL_CSDA_S)[i] = t.S[i];
    C(DP_COL_CSDA_R)[i] = t.R[i];
    C(DP_COL_ION)[i] = t.ion[i];
    C(DP_COL_BREMS)[i] = t.brems[i];
    C(DP_COL_PAIR)[i] = t.pair[i];
    C(DP_COL_PHOTO)[i] = t.photo[i];
  }
  double *S = C(DP_COL_CSDA_S), *T = C(DP_COL_CSDA_T);
  T[0] = 0.0;
  for (int i = 1; i < n; ++i) {
    double K = E[i], Kp = E[i - 1];
    double g = 1.0 + K / mass, gp = 1.0 + Kp / mass;
    double b = std::sqrt(1.0 - 1.0 / (g * g)), bp = std::sqrt(1.0 - 1.0 / (gp * gp));
    double gm = (g + gp) / 2, bm = (b + bp) / 2, sm = (S[i] + S[i - 1]) / 2;
    T[i] = T[i - 1] + (K - Kp) / (sm * bm * gm);
  }
  parallel_for(n, [&](int i) {
    double K = E[i], hard = 0, sg = 0, cs = 0;
    if (K >= 1e-3) {
      for (const auto& e : m.elements) {
        const double f = e.fraction;
        for (int p = 0; p < 4; ++p) hard += f * dcs_moment(p, e.Z, e.A, e.I, mass, K, cut, 1.0, 1);
        sg += f * dcs_moment(P_IONI, e.Z, e.A, e.I, mass, K, 0.0, cut, 2);
      }
      for (const auto& e : m.elements)
        for (int p = 0; p < 4; ++p)
          cs += e.fraction * dcs_moment(p, e.Z, e.A, e.I, mass, K, cut, 1.0, 0);
    }
    C(DP_COL_MIXED_S)[i] = std::max(S[i] - hard, 1e-20);
    C(DP_COL_STRAG)[i] = sg;
    C(DP_COL_XS)[i] = cs;
  });
  double *Sm = C(DP_COL_MIXED_S), *Rm = C(DP_COL_MIXED_R);
  Rm[0] = E[0] / Sm[0];
  for (int i = 1; i < n; ++i) Rm[i] = Rm[i - 1] + (E[i] - E[i - 1]) / ((Sm[i] + Sm[i - 1]) / 2);
  HostMaterial mz = m;
  mz.ZoA = t.ZoA;
  coulomb_and_kinematics(mz, st, n, cols);
}

double host_dcs_moment(int proc, double Z, double A, double I, double mass, double K, double xlo,
                       double xhi, int mode) {
  return dcs_moment(proc, Z, A, I, mass, K, xlo, xhi, mode);
}

}  // namespace dp

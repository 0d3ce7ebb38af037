// coulomb.cpp -- oracle restatement of src/Coulomb.jl: Coulomb scattering
// tables (first transport path, hard elastic path, screening cutoff mu0) from
// Salvat's screened DCS with pole reduction, the KTV Born correction, the
// electronic transverse transport and the radiative soft-scattering
// integrals.  TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <functional>

#include "oracle.hpp"
#include "physics_data.inc"

namespace orc {
namespace {

// src/Coulomb.jl:166-181 (C-index semantics, Rockium = last entry)
double nuclear_radius_c(double Z, double A) {
  int iN = int(Z);
  const int nN = 120;
  if (iN >= nN - 1) iN = nN - 2;
  else if (iN == 1 && A >= 1.5) iN = 0;
  else if (iN == 11 && A == 22.0) iN = nN - 1;
  return DPDATA_NUCLEAR_RADII_FM[iN] * 1e-15;
}

// src/Coulomb.jl:192-206
void frame_parameters(double Z, double A, double mass, double K, double& K0, double& gCM,
                      double& tau) {
  double Ma = Z * PROTON_MASS + (A - Z) * NEUTRON_MASS;
  double M2 = (mass + Ma) * (mass + Ma);
  double s12i = 1.0 / std::sqrt(M2 + 2.0 * Ma * K);
  gCM = (K + mass + Ma) * s12i;
  K0 = (K * Ma + mass * (mass + Ma)) * s12i - mass;
  if (K0 < 1e-9) K0 = 1e-9;
  double etot = K + mass + Ma;
  double b2 = K * (K + 2.0 * mass) / (etot * etot);
  double rM2 = (mass / Ma) * (mass / Ma);
  tau = std::sqrt(rM2 * (1.0 - b2) + b2);
}

// src/Coulomb.jl:211-217
double normalisation(double Z, double A, double mass, double K, double K0) {
  double p2 = K * (K + 2.0 * mass), p02 = K0 * (K0 + 2.0 * mass);
  double d = ALPHA_EM * Z * HBAR_C * (K + mass);
  return A * 1e-3 * p2 * p02 / (d * d * PI * AVOGADRO_NUMBER);
}

struct Screen {
  int n = 0;  // atomic terms + nuclear term
  double amp[4] = {0, 0, 0, 0}, scr[5] = {0, 0, 0, 0, 0};
};

// src/Coulomb.jl:224-289
Screen screening_parameters(double Z, double A, double mass, double K, double K0) {
  double aZE = ALPHA_EM * Z * (K + mass), p2 = K * (K + 2.0 * mass);
  double z2 = aZE * aZE / p2, f;
  if (z2 < 1.0) {
    f = z2 * (1.0 / (1.0 + z2) + 0.20205690315959424 - 0.03692775514336999 * z2 +
              0.008349277381922926 * z2 * z2);
  } else {
    double r2i = 1.0 / (1.0 + z2), phi = -std::atan(std::sqrt(z2));
    f = -0.5 * std::log(r2i) + 0.5 * (1.0 - r2i) + (1.0 / 12.0) * (1.0 - std::cos(2 * phi) * r2i) -
        (1.0 / 120.0) * (1.0 - std::cos(4 * phi) * r2i * r2i) +
        (1.0 / 252.0) * (1.0 - std::cos(6 * phi) * r2i * r2i * r2i);
  }
  double ktv = std::exp(2.0 * f);
  double p02 = K0 * (K0 + 2.0 * mass);
  double d = 0.25 * HBAR_C * HBAR_C / p02 * ktv;
  int iZ = std::min(std::max(int(Z) - 1, 0), 102);
  Screen s;
  int n;
  if (DPDATA_SALVAT_EXPONENT2[iZ] == 1.0) {
    if (iZ == 0) {
      n = 1;
      s.amp[0] = 1.0;
    } else {
      n = 2;
      s.amp[0] = DPDATA_SALVAT_PREFACTOR0[iZ];
      s.amp[1] = 1.0 - s.amp[0];
    }
  } else {
    n = 3;
    s.amp[0] = DPDATA_SALVAT_PREFACTOR0[iZ];
    s.amp[1] = DPDATA_SALVAT_PREFACTOR1[iZ];
    s.amp[2] = 1.0 - (s.amp[0] + s.amp[1]);
  }
  const double* ex[3] = {DPDATA_SALVAT_EXPONENT0, DPDATA_SALVAT_EXPONENT1, DPDATA_SALVAT_EXPONENT2};
  for (int i = 0; i < n; ++i) {
    double a = ex[i][iZ] / BOHR_RADIUS;
    s.scr[i] = d * a * a;
  }
  double RN = nuclear_radius_c(Z, A);
  s.scr[n] = 12.0 * d / (RN * RN);
  s.n = n + 1;
  return s;
}

struct Poles {
  double a[3] = {0, 0, 0}, b[3] = {0, 0, 0}, c[4] = {0, 0, 0, 0};
};

// src/Coulomb.jl:292-348
Poles pole_reduction(const Screen& s) {
  Poles P;
  int n = s.n - 1;
  for (int i = 0; i < n; ++i) {
    double Ai = s.amp[i], Bi = s.scr[i];
    P.b[i] = Ai * Ai;
    for (int j = i + 1; j < n; ++j) {
      double d = 2.0 * Ai * s.amp[j] / (s.scr[j] - Bi);
      P.a[i] += d;
      P.a[j] -= d;
    }
  }
  double N = s.scr[n], Sa[4] = {0, 0, 0, 0}, Sb[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    double x = 1.0 - s.scr[i] / N, r = x;
    for (int j = 0; j < 4; ++j) {
      Sa[j] += P.a[i] / r;
      r *= x;
      Sb[j] += P.b[i] / r;
    }
  }
  double tmp = 1.0;
  for (int i = 0; i < 4; ++i) {
    P.c[i] = ((4 - i) * Sb[3 - i] / N - Sa[3 - i]) * tmp;
    tmp *= N;
  }
  for (int i = 0; i < n; ++i) {
    double Bi = s.scr[i], d = 1.0 - Bi / N, d4 = d * d * d * d;
    P.a[i] = (P.a[i] - 4.0 * P.b[i] / (N - Bi)) / d4;
    P.b[i] = P.b[i] / d4;
  }
  return P;
}

// src/Coulomb.jl:350-406: (cs0, 2*cs1)
void transport_coefficients(double mu, double S, const Screen& s, const Poles& P, double& cs0,
                            double& cs1x2) {
  int n = s.n - 1;
  double c0 = 0, c1 = 0;
  for (int i = 0; i < n; ++i) {
    double al = s.scr[i], r = mu / (mu + al), L = std::log(1.0 + mu / al);
    double I0 = r / al, J0 = L, I1 = L - r, J1 = -al * L, I2 = mu + al * (r - 2.0 * L);
    double J2 = al * (al * L - mu);
    c0 += P.a[i] * (J0 - S * J1) + P.b[i] * (I0 - S * I1);
    c1 += P.a[i] * (J1 - S * J2) + P.b[i] * (I1 - S * I2);
  }
  double N = s.scr[n], r = mu / (mu + N), L = std::log(1.0 + mu / N);
  double I0 = r / N, J0 = L, I1 = L - r, J1 = -N * L, I2 = mu + N * (r - 2.0 * L),
         J2 = N * (N * L - mu);
  double rn = 1.0 / (1.0 + mu / N);
  double K0 = (1.0 - rn) * (1.0 + rn) / (2.0 * N * N);
  double L0 = (1.0 - rn) * ((1.0 + rn) * (1.0 + rn) - rn) / (3.0 * N * N * N);
  double K1 = I0 - N * K0, L1 = K0 - N * L0, K2 = I1 - N * K1, L2 = K1 - N * L1;
  c0 += P.c[0] * (J0 - S * J1) + P.c[1] * (I0 - S * I1) + P.c[2] * (K0 - S * K1) +
        P.c[3] * (L0 - S * L1);
  c1 += P.c[0] * (J1 - S * J2) + P.c[1] * (I1 - S * I2) + P.c[2] * (K1 - S * K2) +
        P.c[3] * (L1 - S * L2);
  cs0 = c0;
  cs1x2 = 2.0 * c1;
}

// src/Coulomb.jl:409-417
double restricted_cs(double mu, double S, const Screen& s, const Poles& P) {
  if (mu >= 1.0 || mu >= 1e6 * s.scr[s.n - 1]) return 0.0;
  double f0, f1, m0, m1;
  transport_coefficients(1.0, S, s, P, f0, f1);
  transport_coefficients(mu, S, s, P, m0, m1);
  return m0 > f0 ? 0.0 : f0 - m0;
}

// src/Coulomb.jl:428-471 (Ridder's method)
double ridder(const std::function<double(double)>& f, double xa, double xb, double fa, double fb,
              double xtol, double rtol, int maxiter) {
  if (fa * fb > 0) return 0.0;
  if (fa == 0) return xa;
  if (fb == 0) return xb;
  double tol = xtol + rtol * std::min(std::fabs(xa), std::fabs(xb)), xn = 0.0;
  for (int it = 0; it < maxiter; ++it) {
    double dm = 0.5 * (xb - xa), xm = xa + dm, fm = f(xm);
    double sgn = fb > fa ? 1.0 : -1.0;
    double dn = sgn * dm * fm / std::sqrt(fm * fm - fa * fb);
    double sgn2 = dn > 0.0 ? 1.0 : -1.0;
    dn = std::fabs(dn);
    double dma = std::fabs(dm) - 0.5 * tol;
    if (dn < dma) dma = dn;
    xn = xm - sgn2 * dma;
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

// src/Coulomb.jl:493-510
double transverse_electronic(double ZoA, double I, double aS, double mass, double K, double nu) {
  double p2 = K * (K + 2.0 * mass), E = K + mass;
  double Wr = 2.0 * ELECTRON_MASS * p2 / (mass * mass + ELECTRON_MASS * (ELECTRON_MASS + 2.0 * E));
  double Wmax = std::min(nu, Wr), b2 = p2 / (E * E);
  double J = std::log(aS * Wmax / I) - b2 * Wmax / Wr + 0.25 * Wmax * Wmax / (E * E) + 1.0 / aS;
  double g = E / mass, lQ = std::log(1.0 + 2.0 * Wr / ELECTRON_MASS);
  double Delta = ALPHA_EM / (2 * PI) * (std::log(2.0 * g) - lQ / 3.0) * lQ * lQ;
  return 2 * PI * ELECTRON_RADIUS * ELECTRON_RADIUS * ELECTRON_MASS * ELECTRON_MASS *
         AVOGADRO_NUMBER * ZoA / (b2 * 1e-3 * p2) * (J + Delta);
}

// src/Coulomb.jl:564-593: integral of theta^2 dsigma/dq over log q, 20-point GL
double transport_integral(double (*dcs)(double, double, double, double, double), double Z,
                          double A, double mass, double K, double qmin, double qmax) {
  if (qmin >= qmax || qmin <= 0.0) return 0.0;
  struct GL20 {
    double x[20], w[20];
    GL20() { gauss_legendre01(20, x, w); }
  };
  static const GL20 g;  // thread-safe one-time initialisation
  double p2 = K * (K + 2.0 * mass), lo = std::log(qmin), hi = std::log(qmax), r = 0.0;
  for (int i = 0; i < 20; ++i) {
    double q = std::exp(lo + (hi - lo) * g.x[i]), v = dcs(Z, A, mass, K, q);
    if (v > 0.0) r += v * (q * q / p2) * q * (g.w[i] * (hi - lo));
  }
  return r;
}

// src/Coulomb.jl:595-635 (mixed-mode soft radiative transport, cutoff fraction)
double radiative_soft(double Z, double A, double mass, double K, double cutoff) {
  const double sqrte = 1.6487212707;
  double qmaxp = K + mass * (1.0 - 0.75 * sqrte * std::pow(Z, 1.0 / 3.0));
  double r = 0.0;
  {
    double qmax = std::min(cutoff * K, qmaxp), qmin = 1e-3 * qmax;
    if (!(qmin >= qmax || qmin <= 0.0))
      r += transport_integral(dcs_bremsstrahlung_ssr, Z, A, mass, K, qmin, qmax);
  }
  {
    double qmax = std::min(cutoff * K, qmaxp), qmin = std::max(4.0 * ELECTRON_MASS, 1e-3 * qmax);
    if (!(qmin >= qmax || qmin <= 0.0))
      r += transport_integral(dcs_pair_production_ssr, Z, A, mass, K, qmin, qmax);
  }
  {
    double qmax = cutoff * K, qmin = std::max(0.0, 1e-3 * qmax);
    if (!(qmin >= qmax || qmin <= 0.0))
      r += transport_integral(dcs_photonuclear_drss, Z, A, mass, K, qmin, qmax);
  }
  return r;
}

}  // namespace

// src/Coulomb.jl:688-826 (compute_coulomb_tables!)
void compute_coulomb_tables(const BaseMaterial& m, double mass, double elastic_ratio,
                            double cutoff, const std::vector<double>& E,
                            const std::vector<double>& csda_R, double ZoA, double I,
                            double density, std::vector<double>& lb1, std::vector<double>& lbe,
                            std::vector<double>& mu0_out) {
  size_t n = E.size();
  double aS = I * 1e9 / (28.816 * std::sqrt(ZoA * density * 1e-3));
  const double max_mu0 = 0.5 * (1.0 - std::cos(1.0 * PI / 180.0));
#pragma omp parallel for schedule(dynamic)
  for (long ii = 0; ii < long(n); ++ii) {
    size_t ie = size_t(ii);
    double K = E[ie];
    if (K <= 0.0) {
      lb1[ie] = lbe[ie] = mu0_out[ie] = 0.0;
      continue;
    }
    size_t ne = m.elements.size();
    std::vector<Screen> sc(ne);
    std::vector<Poles> po(ne);
    std::vector<double> fs(ne), nf(ne), d2(ne);
    double cs_m = 0, cs1_m = 0, A_min = 1e300, cs_A = 0;
    for (size_t k = 0; k < ne; ++k) {
      double Z = m.elements[k].Z, Ae = m.elements[k].A, frac = m.fractions[k];
      double K0, gCM, tau;
      frame_parameters(Z, Ae, mass, K, K0, gCM, tau);
      double e = K + mass;
      fs[k] = K * (e + mass) / (e * e);
      sc[k] = screening_parameters(Z, Ae, mass, K, K0);
      po[k] = pole_reduction(sc[k]);
      double G0, G1;
      transport_coefficients(1.0, fs[k], sc[k], po[k], G0, G1);
      nf[k] = frac / normalisation(Z, Ae, mass, K, K0);
      cs_m += nf[k] * G0;
      double d = 1.0 / (gCM * (1.0 + tau));
      d2[k] = d * d;
      cs1_m += nf[k] * G1 * d2[k];
      for (int j = 0; j < sc[k].n - 1; ++j) A_min = std::min(A_min, sc[k].scr[j]);
      cs_A += nf[k];
    }
    cs_A /= A_min * (A_min + 1.0);
    double range_i = csda_R[ie] > 0.0 ? 1.0 / csda_R[ie] : 0.0;
    double cs_h = std::max(cs1_m, range_i) / elastic_ratio;
    if (cs_h < 1.0 / EHS_PATH_MAX) cs_h = 1.0 / EHS_PATH_MAX;
    double mu0, lb_h;
    if (cs_h < cs_m) {
      double zeta = cs_h / cs_A;
      double mu_max = A_min * (1.0 - zeta) / (A_min + zeta);
      if (mu_max > max_mu0) mu_max = max_mu0;
      auto obj = [&](double mu) {
        double t = 0;
        for (size_t k = 0; k < ne; ++k) t += nf[k] * restricted_cs(mu, fs[k], sc[k], po[k]);
        return t - cs_h;
      };
      double fmax = obj(mu_max), fmin = cs_m - cs_h;
      mu0 = ridder(obj, 0.0, mu_max, fmin, fmax, 1e-6 * mu_max, 1e-6, 100);
      if (mu0 > max_mu0) mu0 = max_mu0;
      cs_h += obj(mu0);
      lb_h = cs_h <= 1.0 / EHS_PATH_MAX ? EHS_PATH_MAX : 1.0 / cs_h;
    } else {
      mu0 = 0.0;
      lb_h = 1.0 / cs_m;
    }
    mu0_out[ie] = mu0;
    lbe[ie] = lb_h * K * (K + 2.0 * mass);
    double inv = 0;
    for (size_t k = 0; k < ne; ++k) {
      double G0, G1;
      transport_coefficients(mu0, fs[k], sc[k], po[k], G0, G1);
      inv += nf[k] * d2[k] * G1;
    }
    double rad = 0;
    for (size_t k = 0; k < ne; ++k)
      rad += radiative_soft(m.elements[k].Z, m.elements[k].A, mass, K, cutoff) * m.fractions[k];
    double el = transverse_electronic(ZoA, I, aS, mass, K, cutoff * K);
    double tot = inv + rad + el;
    lb1[ie] = tot > 0.0 ? 1.0 / tot : 0.0;
  }
}

}  // namespace orc

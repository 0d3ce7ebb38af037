// dcs.cuh -- differential cross sections of the muon hard processes, usable
// on host (table building) and device (adjoint hard events).  Restates
// src/Materials.jl:513-926: SSR bremsstrahlung, SSR pair production (12-point
// Gauss-Legendre over the pair asymmetry), DRSS photonuclear with the ALLM97
// structure function (9-point Gauss-Legendre in log Q^2) and Salvat's
// close-collision ionisation DCS.  Returns dsigma/dq per atom in m^2/GeV.
#pragma once
#include "common.cuh"

namespace dp {

// Gauss-Legendre nodes/weights on [0, 1] (computed by Newton iteration).
DP_HD double gl9(int i, bool weight) {
  const double x[9] = {0.015919880246186957, 0.08198444633668206, 0.19331428364970477,
                       0.33787328829809554,  0.5,                 0.66212671170190451,
                       0.80668571635029518,  0.91801555366331788, 0.98408011975381304};
  const double w[9] = {0.040637194180787317, 0.090324080347428781, 0.13030534820146777,
                       0.15617353852000146,  0.16511967750062989,  0.15617353852000146,
                       0.13030534820146777,  0.090324080347428781, 0.040637194180787317};
  return weight ? w[i] : x[i];
}
DP_HD double gl12(int i, bool weight) {
  const double x[12] = {0.0092196828766403782, 0.047941371814762601, 0.11504866290284765,
                        0.20634102285669126,   0.31608425050090994,  0.43738329574426554,
                        0.5626167042557344,    0.68391574949909006,  0.79365897714330869,
                        0.88495133709715235,   0.95205862818523745,  0.99078031712335957};
  const double w[12] = {0.023587668193255917, 0.053469662997659088, 0.080039164271673166,
                        0.10158371336153292,  0.11674626826917739,  0.12457352290670144,
                        0.12457352290670144,  0.11674626826917739,  0.10158371336153292,
                        0.080039164271673166, 0.053469662997659088, 0.023587668193255917};
  return weight ? w[i] : x[i];
}

// Real dilogarithm for x <= 1 (Bernoulli series in -log(1-x) plus the
// reflection Li2(x) = pi^2/6 - log x log(1-x) - Li2(1-x)).  The DCS only
// evaluates it on (0, 1).
DP_HD double li2_bernoulli(double x) {
  double u = -log1p(-x);
  double u2 = u * u;
  // B_n/(n+1)! for n = 2, 4, ..., 20 (odd n > 1 vanish)
  const double c[10] = {1.0 / 36.0, -1.0 / 3600.0, 1.0 / 211680.0, -1.0 / 10886400.0,
                        1.0 / 526901760.0, -4.064761645144225e-11, 8.921691020456453e-13,
                        -1.9939295860721077e-14, 4.5189800296199183e-16, -1.0356517612181247e-17};
  double s = 0.0, p = u * u2;
  for (int k = 0; k < 10; ++k) {
    s += c[k] * p;
    p *= u2;
  }
  return u - 0.25 * u2 + s;
}
DP_HD double dilog(double x) {
  const double pi2_6 = kPi * kPi / 6.0;
  if (x == 1.0) return pi2_6;
  if (x <= 0.5) return li2_bernoulli(x);
  return pi2_6 - log(x) * log1p(-x) - li2_bernoulli(1.0 - x);
}

// src/Materials.jl:576-620
DP_HD double radiation_log(double Z) {
  switch (int(Z + 0.5)) {
    case 1: return 202.4;  case 2: return 151.9;  case 3: return 159.9;  case 4: return 172.3;
    case 5: return 177.9;  case 6: return 178.3;  case 7: return 176.6;  case 8: return 173.4;
    case 9: return 170.0;  case 10: return 165.8; case 11: return 165.8; case 12: return 167.1;
    case 13: return 169.1; case 14: return 170.8; case 15: return 172.2; case 16: return 173.4;
    case 17: return 174.3; case 18: return 174.8; case 19: return 175.1; case 20: return 175.6;
    case 21: return 176.2; case 22: return 176.8; case 26: return 175.8; case 29: return 173.1;
    case 32: return 173.0; case 35: return 173.5; case 42: return 175.9; case 50: return 177.4;
    case 53: return 178.6; case 74: return 177.6; case 82: return 178.0; case 92: return 179.8;
    default: return 182.7;
  }
}

constexpr double kSqrtE = 1.648721270700128;
constexpr double kMeMeV = 0.5109989461;
constexpr double kReCm = 2.8179403227e-13;
constexpr double kMmuMeV = 105.6583745;

// src/Materials.jl:631-695
DP_HD double dcs_brems(double Z, double A, double m, double K, double q) {
  if (Z <= 0 || A <= 0 || m <= 0 || K <= 0 || q <= 0) return 0.0;
  double z13 = pow(Z, 1.0 / 3.0);
  if (q >= K + m * (1.0 - 0.75 * kSqrtE * z13)) return 0.0;
  double energy = (K + m) * 1e3, v = q * 1e3 / energy, mm = m * 1e3, Zi13 = 1.0 / z13;
  double rl = radiation_log(Z), rli = Z == 1.0 ? 446.0 : 1429.0;
  double Dn = 1.54 * pow(A, 0.27);
  double mu = mm / (kMmuMeV * exp(1.0) / Dn);
  double rho = sqrt(1.0 + 4.0 * mu * mu);
  double lr = log((rho + 1.0) / (rho - 1.0));
  double d1 = log(mu) + 0.5 * rho * lr;
  double d2 = log(mu) + 0.25 * (3.0 * rho - rho * rho * rho) * lr + 2.0 * mu * mu;
  double delta = mm * mm * v / (2.0 * energy * (1.0 - v));
  double phi1 = log(rl * Zi13 * (mm / kMeMeV) / (1.0 + rl * Zi13 * exp(0.5) * delta / kMeMeV));
  double phi2 = log(rl * Zi13 * exp(-1.0 / 6.0) * (mm / kMeMeV) /
                    (1.0 + rl * Zi13 * exp(1.0 / 3.0) * delta / kMeMeV));
  phi1 -= d1 * (1.0 - 1.0 / Z);
  phi2 -= d2 * (1.0 - 1.0 / Z);
  double sa = (4.0 / 3.0 * (1.0 - v) + v * v) *
              (log(mm / delta / (mm * delta / (kMeMeV * kMeMeV) + kSqrtE)) -
               log(1.0 + kMeMeV / (delta * rli * Zi13 * Zi13 * kSqrtE)));
  double sr;
  if (v < 0.0 || v > 1.0) {
    sr = 0.0;
  } else if (v < 0.02) {
    sr = -0.00349 + 148.84 * v - 987.531 * v * v;
  } else if (v < 0.1) {
    sr = 0.1642 + 132.573 * v - 585.361 * v * v + 1407.77 * v * v * v;
  } else if (v < 0.9) {
    double t = log(1.0 - v);
    sr = -2.8922 - 19.0156 * v + 57.698 * v * v - 63.418 * v * log(v) + 14.1166 * t + 1.84206 * t * t;
  } else {
    double t = log(1.0 - v);
    sr = 2134.19 + 581.823 * v - 2708.85 * v * v + 4767.05 * v * log(v) + 1.52918 * t + 0.361933 * t * t;
  }
  double r = ((2.0 - 2.0 * v + v * v) * phi1 - 2.0 / 3.0 * (1.0 - v) * phi2) + sa / Z +
             0.25 * kAlpha * phi1 * sr;
  if (r <= 0.0) return 0.0;
  double aux = 2.0 * (kMeMeV / mm) * kReCm * Z;
  return aux * aux * (kAlpha / q) * r * 1e-4;
}

// src/Materials.jl:701-800: d2 sigma / (dq drho) of the SSR pair model.
DP_HD double pair_d2(double Z, double A, double mass, double K, double q, double rho_in) {
  double energy = (K + mass) * 1e3, v = q / (K + mass), m = mass * 1e3;
  double rl = radiation_log(Z);
  double cpf = 4.0 / (3.0 * kPi) * Z * (kAlpha * kReCm) * (kAlpha * kReCm);
  double Z13 = pow(Z, -1.0 / 3.0), dn = 1.54 * pow(A, 0.27);
  double rho = 1.0 - rho_in, r2 = rho * rho;
  double g1 = Z == 1.0 ? 4.4e-5 : 1.95e-5, g2 = Z == 1.0 ? 4.8e-5 : 5.3e-5;
  double z1 = 0.073 * log(energy / m / (1.0 + g1 * pow(Z, 2.0 / 3.0) * energy / m)) - 0.26;
  double z2 = 0.058 * log(energy / m / (1.0 + g2 / Z13 * energy / m)) - 0.14;
  double zeta = (z1 > 0.0 && z2 > 0.0) ? z1 / z2 : 0.0;
  double beta = v * v / (2.0 * (1.0 - v));
  double xi = (m * v / (2.0 * kMeMeV)) * (m * v / (2.0 * kMeMeV)) * (1.0 - r2) / (1.0 - v);
  double lxi = log(1.0 + 1.0 / xi), l1x = log(1.0 + xi);
  double den = energy * v * (1.0 - r2);
  double mdn2 = (kMeMeV / m * dn) * (kMeMeV / m * dn);
  double Be = ((2.0 + r2) * (1.0 + beta) + xi * (3.0 + r2)) * lxi + (1.0 - r2 - beta) / (1.0 + xi) -
              (3.0 + r2);
  double Ce2 = ((1.0 - r2) * (1.0 + beta) + xi * (3.0 - r2)) * lxi +
               2.0 * (1.0 - beta - r2) / (1.0 + xi) - (3.0 - r2);
  double Ce1 = Be - Ce2;
  double De = ((2.0 + r2) * (1.0 + beta) + xi * (3.0 + r2)) * dilog(1.0 / (1.0 + xi)) -
              (2.0 + r2) * xi * lxi - (xi + r2 + beta) / (1.0 + xi);
  double Le1, Le2, t = De / Be;
  if (t > 0.0) {
    double X = t < 100.0 ? exp(-t) : 0.0;
    Le1 = log(rl * Z13 * sqrt(1.0 + xi) / (X + 2.0 * kMeMeV * exp(0.5) * rl * Z13 * (1.0 + xi) / den)) -
          t - 0.5 * log(X + mdn2 * (1.0 + xi));
    Le2 = log(rl * Z13 * exp(-1.0 / 6.0) * sqrt(1.0 + xi) /
              (X + 2.0 * kMeMeV * exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den)) -
          t - 0.5 * log(X + mdn2 * exp(-1.0 / 3.0) * (1.0 + xi));
  } else {
    double X = t > -100.0 ? exp(t) : 0.0;
    Le1 = log(rl * Z13 * sqrt(1.0 + xi) /
              (1.0 + X * 2.0 * kMeMeV * exp(0.5) * rl * Z13 * (1.0 + xi) / den)) -
          0.5 * t - 0.5 * log(1.0 + X * mdn2 * (1.0 + xi));
    Le2 = log(rl * Z13 * exp(-1.0 / 6.0) * sqrt(1.0 + xi) /
              (1.0 + X * 2.0 * kMeMeV * exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den)) -
          0.5 * t - 0.5 * log(1.0 + X * mdn2 * exp(-1.0 / 3.0) * (1.0 + xi));
  }
  double de = cpf * (Z + zeta) * (1.0 - v) / v * (Ce1 * Le1 + Ce2 * Le2);
  if (de < 0.0) de = 0.0;
  double bb = (1.0 + r2) * (1.0 + 1.5 * beta) - 1.0 / xi * (1.0 + 2.0 * beta) * (1.0 - r2);
  double Bm = bb * l1x + xi * (1.0 - r2 - beta) / (1.0 + xi) + (1.0 + 2.0 * beta) * (1.0 - r2);
  double Cm2 = ((1.0 - beta) * (1.0 - r2) - xi * (1.0 + r2)) * l1x / xi -
               2.0 * (1.0 - beta - r2) / (1.0 + xi) + 1.0 - beta - (1.0 + beta) * r2;
  double Cm1 = Bm - Cm2;
  double Dm = bb * dilog(xi / (1.0 + xi)) + (1.0 + 1.5 * beta) * (1.0 - r2) / xi * l1x +
              (1.0 - r2 - 0.5 * beta * (1.0 + r2) + (1.0 - r2) / (2.0 * xi) * beta) * xi / (1.0 + xi);
  double Lm1, Lm2, s = Dm / Bm;
  double pre = m / kMeMeV * rl * Z13 / dn;
  if (s > 0.0) {
    double X = s < 100.0 ? exp(-s) : 0.0;
    Lm1 = log(pre / (X + 2.0 * kMeMeV * exp(0.5) * rl * Z13 * (1.0 + xi) / den)) - s;
    Lm2 = log(pre / (X + 2.0 * kMeMeV * exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den)) - s;
  } else {
    double X = s > -100.0 ? exp(s) : 0.0;
    Lm1 = log(pre / (1.0 + 2.0 * kMeMeV * exp(0.5) * rl * Z13 * (1.0 + xi) / den * X));
    Lm2 = log(pre / (1.0 + 2.0 * kMeMeV * exp(1.0 / 3.0) * rl * Z13 * (1.0 + xi) / den * X));
  }
  double dm = cpf * (Z + zeta) * (1.0 - v) / v * (kMeMeV / m) * (kMeMeV / m) * (Cm1 * Lm1 + Cm2 * Lm2);
  if (dm < 0.0) dm = 0.0;
  return (de + dm) * 0.1 / energy;
}

// src/Materials.jl:802-832
DP_HD double dcs_pair(double Z, double A, double mass, double K, double q) {
  if (Z <= 0 || A <= 0 || mass <= 0 || K <= 0 || q <= 0) return 0.0;
  if (q <= 4.0 * kElectronMass) return 0.0;
  if (q >= K + mass * (1.0 - 0.75 * 1.6487212707 * pow(Z, 1.0 / 3.0))) return 0.0;
  double gamma = 1.0 + K / mass;
  double x0 = 1.0 - 4.0 * kElectronMass / q, x1 = 1.0 - 6.0 / (gamma * (gamma - q / mass));
  if (!(x0 > 0.0 && x1 > 0.0)) return 0.0;
  double ri = 1.0 - sqrt(x0) * x1;
  if (ri <= 0.0 || ri >= 1.0) return 0.0;
  double tmin = log(ri), I = 0.0;
  for (int i = 0; i < 12; ++i) {
    double r = exp(gl12(i, false) * tmin);
    I -= pair_d2(Z, A, mass, K, q, r) * r * gl12(i, true) * tmin;
  }
  return I < 0.0 ? 0.0 : I;
}

// src/Materials.jl:838-926
DP_HD double f2p_allm97(double x, double Q2) {
  const double m02 = 0.31985, mP2 = 49.457, mR2 = 0.15052, Q02 = 0.52544, L2 = 0.06527;
  double M = 0.5 * (kProtonMass + kNeutronMass), M2 = M * M;
  double W2 = M2 + Q2 * (1.0 / x - 1.0);
  double t = log(log((Q2 + Q02) / L2) / log(Q02 / L2));
  double xP = (Q2 + mP2) / (Q2 + mP2 + W2 - M2), xR = (Q2 + mR2) / (Q2 + mR2 + W2 - M2);
  double cP = 0.28067 + (0.28067 - 0.22291) * (1.0 / (1.0 + pow(t, 2.1979)) - 1.0);
  double aP = -0.0808 + (-0.0808 + 0.44812) * (1.0 / (1.0 + pow(t, 1.1709)) - 1.0);
  double bP = 0.36292 + 1.8917 * pow(t, 1.8439);
  double cR = 0.80107 + 0.97307 * pow(t, 3.4942);
  double aR = 0.58400 + 0.37888 * pow(t, 2.6063);
  double bR = 0.01147 + 3.7582 * pow(t, 0.49338);
  double F2P = cP * exp(aP * log(xP) + bP * log(1.0 - x));
  double F2R = cR * exp(aR * log(xR) + bR * log(1.0 - x));
  return Q2 / (Q2 + m02) * (F2P + F2R);
}
DP_HD double photo_d2(double Z, double A, double ml, double K, double q, double Q2) {
  double cf = 4.0 * kPi * kAlpha * kAlpha * kHbarC * kHbarC;
  double M = 0.5 * (kProtonMass + kNeutronMass), E = K + ml, y = q / E, x = 0.5 * Q2 / (M * q);
  double F2p = f2p_allm97(x, Q2);
  double sh = 1.0;
  if (Z != 1.0) {
    if (x < 0.0014) sh = exp(-0.1 * log(A));
    else if (x < 0.04) sh = exp((0.069 * log10(x) + 0.097) * log(A));
  }
  double F2A = F2p * sh * (Z + (A - Z) * (1.0 + x * (-1.85 + x * (2.45 + x * (-2.35 + x)))));
  double dds = (1.0 - y + 0.5 * (1.0 - 2.0 * ml * ml / Q2) * (y * y + Q2 / (E * E))) / (Q2 * Q2) -
               0.25 / (E * E * Q2);
  return cf * F2A * dds / q;
}
DP_HD double dcs_photo(double Z, double A, double m, double K, double q) {
  if (Z <= 0 || A <= 0 || m <= 0 || K <= 0 || q <= 0) return 0.0;
  double M = 0.5 * (kNeutronMass + kProtonMass), mpi = kPionMass;
  if (q <= mpi + 0.5 * mpi * mpi / M || q >= K + m - 0.5 * (M + m * m / M)) return 0.0;
  double E = K + m, ml2 = m * m;
  double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
  double Q2max = 2.0 * M * (q - mpi) - mpi * mpi;
  if (Q2max < Q2min || Q2min < 0.0) return 0.0;
  double lmin = log(Q2min), dx = log(Q2max) - lmin, ds = 0.0;
  for (int i = 0; i < 9; ++i) {
    double Q2 = exp(lmin + dx * gl9(i, false));
    double v = photo_d2(Z, A, m, K, q, Q2);
    if (v > 0.0) ds += v * (gl9(i, true) * dx * Q2);
  }
  return ds < 0.0 ? 0.0 : ds;
}

// src/Materials.jl:513-528
DP_HD double dcs_ionisation(double Z, double I, double m, double K, double q) {
  double P2 = K * (K + 2.0 * m), E = K + m;
  double Wmax = 2.0 * kElectronMass * P2 / (m * m + kElectronMass * (kElectronMass + 2.0 * E));
  if (q > Wmax) return 0.0;
  if (q <= (13.6 / 19.2) * I) return 0.0;
  double E2 = E * E, b2 = P2 / E2;
  return 2.0 * kPi * kElectronMass * kElectronRadius * kElectronRadius * Z *
         (0.5 / E2 + 1.0 / q * (1.0 / q - b2 / Wmax)) / b2;
}

}  // namespace dp

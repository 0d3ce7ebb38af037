// dcs.cuh -- differential cross sections of the muon hard processes, usable
// on host (table building) and device (adjoint hard events).  Restates
// src/Materials.jl:513-926: SSR bremsstrahlung, SSR pair production (12-point
// Gauss-Legendre over the pair asymmetry), DRSS photonuclear with the ALLM97
// structure function (9-point Gauss-Legendre in log Q^2) and Salvat's
// close-collision ionisation DCS.  Returns dsigma/dq per atom in m^2/GeV.
#pragma once
#include "common.cuh"

namespace dp {

// Gauss-Legendre nodes/weights on [0, 1] (computed by Newton iteration): 9
// nodes then 9 weights, 12 nodes then 12 weights.  On the device the terms
// read them from global tables; a function-local table indexed at run time
// is built in each thread's local memory at every call.  The FP32 tables hold
// the float of each FP64 entry.
#define DP_GL9 \
    0.015919880246186957, 0.08198444633668206, 0.19331428364970477, \
    0.33787328829809554, 0.5, 0.66212671170190451, \
    0.80668571635029518, 0.91801555366331788, 0.98408011975381304, \
    0.040637194180787317, 0.090324080347428781, 0.13030534820146777, \
    0.15617353852000146, 0.16511967750062989, 0.15617353852000146, \
    0.13030534820146777, 0.090324080347428781, 0.040637194180787317
#define DP_GL12 \
    0.0092196828766403782, 0.047941371814762601, 0.11504866290284765, \
    0.20634102285669126, 0.31608425050090994, 0.43738329574426554, \
    0.5626167042557344, 0.68391574949909006, 0.79365897714330869, \
    0.88495133709715235, 0.95205862818523745, 0.99078031712335957, \
    0.023587668193255917, 0.053469662997659088, 0.080039164271673166, \
    0.10158371336153292, 0.11674626826917739, 0.12457352290670144, \
    0.12457352290670144, 0.11674626826917739, 0.10158371336153292, \
    0.080039164271673166, 0.053469662997659088, 0.023587668193255917
__device__ const double kGl9d[18] = {DP_GL9};
__device__ const double kGl12d[24] = {DP_GL12};
__device__ const float kGl9f[18] = {
    float(0.015919880246186957), float(0.08198444633668206), float(0.19331428364970477),
    float(0.33787328829809554), float(0.5), float(0.66212671170190451),
    float(0.80668571635029518), float(0.91801555366331788), float(0.98408011975381304),
    float(0.040637194180787317), float(0.090324080347428781), float(0.13030534820146777),
    float(0.15617353852000146), float(0.16511967750062989), float(0.15617353852000146),
    float(0.13030534820146777), float(0.090324080347428781), float(0.040637194180787317),
};
__device__ const float kGl12f[24] = {
    float(0.0092196828766403782), float(0.047941371814762601), float(0.11504866290284765),
    float(0.20634102285669126), float(0.31608425050090994), float(0.43738329574426554),
    float(0.5626167042557344), float(0.68391574949909006), float(0.79365897714330869),
    float(0.88495133709715235), float(0.95205862818523745), float(0.99078031712335957),
    float(0.023587668193255917), float(0.053469662997659088), float(0.080039164271673166),
    float(0.10158371336153292), float(0.11674626826917739), float(0.12457352290670144),
    float(0.12457352290670144), float(0.11674626826917739), float(0.10158371336153292),
    float(0.080039164271673166), float(0.053469662997659088), float(0.023587668193255917),
};
DP_HD double gl9(int i, bool weight) {
#ifdef __CUDA_ARCH__
  return kGl9d[(weight ? 9 : 0) + i];
#else
  static const double t[18] = {DP_GL9};
  return t[(weight ? 9 : 0) + i];
#endif
}
DP_HD double gl12(int i, bool weight) {
#ifdef __CUDA_ARCH__
  return kGl12d[(weight ? 12 : 0) + i];
#else
  static const double t[24] = {DP_GL12};
  return t[(weight ? 12 : 0) + i];
#endif
}
#undef DP_GL9
#undef DP_GL12
template <class T>
DP_HD T gl9_t(int i, bool weight) {
#ifdef __CUDA_ARCH__
  if constexpr (sizeof(T) == 4) return kGl9f[(weight ? 9 : 0) + i];
#endif
  return T(gl9(i, weight));
}
template <class T>
DP_HD T gl12_t(int i, bool weight) {
#ifdef __CUDA_ARCH__
  if constexpr (sizeof(T) == 4) return kGl12f[(weight ? 12 : 0) + i];
#endif
  return T(gl12(i, weight));
}

// Real dilogarithm for x <= 1 (Bernoulli series in -log(1-x) plus the
// reflection Li2(x) = pi^2/6 - log x log(1-x) - Li2(1-x)).  The DCS only
// evaluates it on (0, 1).
template <class T>
DP_HD T li2_bernoulli(T x) {
  T u = -log1p(-x);
  T u2 = u * u;
  // B_n/(n+1)! for n = 2, 4, ..., 20 (odd n > 1 vanish)
  const double c[10] = {1.0 / 36.0, -1.0 / 3600.0, 1.0 / 211680.0, -1.0 / 10886400.0,
                        1.0 / 526901760.0, -4.064761645144225e-11, 8.921691020456453e-13,
                        -1.9939295860721077e-14, 4.5189800296199183e-16, -1.0356517612181247e-17};
  T s = T(0), p = u * u2;
#pragma unroll  // the coefficients fold to constants of T (no FP64 conversion per term)
  for (int k = 0; k < 10; ++k) {
    s += T(c[k]) * p;
    p *= u2;
  }
  return u - T(0.25) * u2 + s;
}
template <class T>
DP_HD T dilog(T x) {
  const T pi2_6 = T(kPi * kPi / 6.0);
  if (x == T(1)) return pi2_6;
  if (x <= T(0.5)) return li2_bernoulli(x);
  return pi2_6 - log(x) * log1p(-x) - li2_bernoulli(T(1) - x);
}

// src/Materials.jl:576-620
template <class T>
DP_HD T radiation_log(T Z) {
  switch (int(Z + T(0.5))) {
    case 1: return T(202.4);  case 2: return T(151.9);  case 3: return T(159.9);  case 4: return T(172.3);
    case 5: return T(177.9);  case 6: return T(178.3);  case 7: return T(176.6);  case 8: return T(173.4);
    case 9: return T(170.0);  case 10: return T(165.8); case 11: return T(165.8); case 12: return T(167.1);
    case 13: return T(169.1); case 14: return T(170.8); case 15: return T(172.2); case 16: return T(173.4);
    case 17: return T(174.3); case 18: return T(174.8); case 19: return T(175.1); case 20: return T(175.6);
    case 21: return T(176.2); case 22: return T(176.8); case 26: return T(175.8); case 29: return T(173.1);
    case 32: return T(173.0); case 35: return T(173.5); case 42: return T(175.9); case 50: return T(177.4);
    case 53: return T(178.6); case 74: return T(177.6); case 82: return T(178.0); case 92: return T(179.8);
    default: return T(182.7);
  }
}

constexpr double kSqrtE = 1.648721270700128;
constexpr double kMeMeV = 0.5109989461;
constexpr double kReCm = 2.8179403227e-13;
constexpr double kMmuMeV = 105.6583745;

// The DCS below take a `scale` multiplying the result (1 for the per-atom
// value in m^2/GeV).  The FP32 instantiations pass N_A/(A 1e-3) so that the
// per-mass value stays far from the FP32 underflow.

// src/Materials.jl:631-695
template <class T>
DP_HD T dcs_brems(T Z, T A, T m, T K, T q, T scale = T(1)) {
  if (Z <= T(0) || A <= T(0) || m <= T(0) || K <= T(0) || q <= T(0)) return T(0);
  T z13 = pow(Z, T(1) / T(3));
  if (q >= K + m * (T(1) - T(0.75) * T(kSqrtE) * z13)) return T(0);
  T energy = (K + m) * T(1e3), v = q * T(1e3) / energy, mm = m * T(1e3), Zi13 = T(1) / z13;
  T rl = radiation_log(Z), rli = Z == T(1) ? T(446.0) : T(1429.0);
  T Dn = T(1.54) * pow(A, T(0.27));
  T mu = mm / (T(kMmuMeV) * exp(T(1)) / Dn);
  T rho = sqrt(T(1) + T(4) * mu * mu);
  T lr = log((rho + T(1)) / (rho - T(1)));
  T d1 = log(mu) + T(0.5) * rho * lr;
  T d2 = log(mu) + T(0.25) * (T(3) * rho - rho * rho * rho) * lr + T(2) * mu * mu;
  T delta = mm * mm * v / (T(2) * energy * (T(1) - v));
  T phi1 = log(rl * Zi13 * (mm / T(kMeMeV)) / (T(1) + rl * Zi13 * exp(T(0.5)) * delta / T(kMeMeV)));
  T phi2 = log(rl * Zi13 * exp(T(-1) / T(6)) * (mm / T(kMeMeV)) /
               (T(1) + rl * Zi13 * exp(T(1) / T(3)) * delta / T(kMeMeV)));
  phi1 -= d1 * (T(1) - T(1) / Z);
  phi2 -= d2 * (T(1) - T(1) / Z);
  T sa = (T(4) / T(3) * (T(1) - v) + v * v) *
         (log(mm / delta / (mm * delta / (T(kMeMeV) * T(kMeMeV)) + T(kSqrtE))) -
          log(T(1) + T(kMeMeV) / (delta * rli * Zi13 * Zi13 * T(kSqrtE))));
  T sr;
  if (v < T(0) || v > T(1)) {
    sr = T(0);
  } else if (v < T(0.02)) {
    sr = T(-0.00349) + T(148.84) * v - T(987.531) * v * v;
  } else if (v < T(0.1)) {
    sr = T(0.1642) + T(132.573) * v - T(585.361) * v * v + T(1407.77) * v * v * v;
  } else if (v < T(0.9)) {
    T t = log(T(1) - v);
    sr = T(-2.8922) - T(19.0156) * v + T(57.698) * v * v - T(63.418) * v * log(v) + T(14.1166) * t +
         T(1.84206) * t * t;
  } else {
    T t = log(T(1) - v);
    sr = T(2134.19) + T(581.823) * v - T(2708.85) * v * v + T(4767.05) * v * log(v) + T(1.52918) * t +
         T(0.361933) * t * t;
  }
  T r = ((T(2) - T(2) * v + v * v) * phi1 - T(2) / T(3) * (T(1) - v) * phi2) + sa / Z +
        T(0.25) * T(kAlpha) * phi1 * sr;
  if (r <= T(0)) return T(0);
  T aux = T(2) * (T(kMeMeV) / mm) * T(kReCm) * Z;
  return aux * aux * scale * (T(kAlpha) / q) * r * T(1e-4);
}

// src/Materials.jl:701-800: d2 sigma / (dq drho) of the SSR pair model.
template <class T>
DP_HD T pair_d2(T Z, T A, T mass, T K, T q, T rho_in, T scale = T(1)) {
  T energy = (K + mass) * T(1e3), v = q / (K + mass), m = mass * T(1e3);
  T rl = radiation_log(Z);
  T cpf = T(4) / (T(3) * T(kPi)) * Z * (T(kAlpha) * T(kReCm)) * (T(kAlpha) * T(kReCm)) * scale;
  T Z13 = pow(Z, T(-1) / T(3)), dn = T(1.54) * pow(A, T(0.27));
  T rho = T(1) - rho_in, r2 = rho * rho;
  T g1 = Z == T(1) ? T(4.4e-5) : T(1.95e-5), g2 = Z == T(1) ? T(4.8e-5) : T(5.3e-5);
  T z1 = T(0.073) * log(energy / m / (T(1) + g1 * pow(Z, T(2) / T(3)) * energy / m)) - T(0.26);
  T z2 = T(0.058) * log(energy / m / (T(1) + g2 / Z13 * energy / m)) - T(0.14);
  T zeta = (z1 > T(0) && z2 > T(0)) ? z1 / z2 : T(0);
  T beta = v * v / (T(2) * (T(1) - v));
  T xi = (m * v / (T(2) * T(kMeMeV))) * (m * v / (T(2) * T(kMeMeV))) * (T(1) - r2) / (T(1) - v);
  T lxi = log(T(1) + T(1) / xi), l1x = log(T(1) + xi);
  T den = energy * v * (T(1) - r2);
  T mdn2 = (T(kMeMeV) / m * dn) * (T(kMeMeV) / m * dn);
  T Be = ((T(2) + r2) * (T(1) + beta) + xi * (T(3) + r2)) * lxi + (T(1) - r2 - beta) / (T(1) + xi) -
         (T(3) + r2);
  T Ce2 = ((T(1) - r2) * (T(1) + beta) + xi * (T(3) - r2)) * lxi +
          T(2) * (T(1) - beta - r2) / (T(1) + xi) - (T(3) - r2);
  T Ce1 = Be - Ce2;
  T De = ((T(2) + r2) * (T(1) + beta) + xi * (T(3) + r2)) * dilog(T(1) / (T(1) + xi)) -
         (T(2) + r2) * xi * lxi - (xi + r2 + beta) / (T(1) + xi);
  T Le1, Le2, t = De / Be;
  if (t > T(0)) {
    T X = t < T(100) ? exp(-t) : T(0);
    Le1 = log(rl * Z13 * sqrt(T(1) + xi) / (X + T(2) * T(kMeMeV) * exp(T(0.5)) * rl * Z13 * (T(1) + xi) / den)) -
          t - T(0.5) * log(X + mdn2 * (T(1) + xi));
    Le2 = log(rl * Z13 * exp(T(-1) / T(6)) * sqrt(T(1) + xi) /
              (X + T(2) * T(kMeMeV) * exp(T(1) / T(3)) * rl * Z13 * (T(1) + xi) / den)) -
          t - T(0.5) * log(X + mdn2 * exp(T(-1) / T(3)) * (T(1) + xi));
  } else {
    T X = t > T(-100) ? exp(t) : T(0);
    Le1 = log(rl * Z13 * sqrt(T(1) + xi) /
              (T(1) + X * T(2) * T(kMeMeV) * exp(T(0.5)) * rl * Z13 * (T(1) + xi) / den)) -
          T(0.5) * t - T(0.5) * log(T(1) + X * mdn2 * (T(1) + xi));
    Le2 = log(rl * Z13 * exp(T(-1) / T(6)) * sqrt(T(1) + xi) /
              (T(1) + X * T(2) * T(kMeMeV) * exp(T(1) / T(3)) * rl * Z13 * (T(1) + xi) / den)) -
          T(0.5) * t - T(0.5) * log(T(1) + X * mdn2 * exp(T(-1) / T(3)) * (T(1) + xi));
  }
  T de = cpf * (Z + zeta) * (T(1) - v) / v * (Ce1 * Le1 + Ce2 * Le2);
  if (de < T(0)) de = T(0);
  T bb = (T(1) + r2) * (T(1) + T(1.5) * beta) - T(1) / xi * (T(1) + T(2) * beta) * (T(1) - r2);
  T Bm = bb * l1x + xi * (T(1) - r2 - beta) / (T(1) + xi) + (T(1) + T(2) * beta) * (T(1) - r2);
  T Cm2 = ((T(1) - beta) * (T(1) - r2) - xi * (T(1) + r2)) * l1x / xi -
          T(2) * (T(1) - beta - r2) / (T(1) + xi) + T(1) - beta - (T(1) + beta) * r2;
  T Cm1 = Bm - Cm2;
  T Dm = bb * dilog(xi / (T(1) + xi)) + (T(1) + T(1.5) * beta) * (T(1) - r2) / xi * l1x +
         (T(1) - r2 - T(0.5) * beta * (T(1) + r2) + (T(1) - r2) / (T(2) * xi) * beta) * xi / (T(1) + xi);
  T Lm1, Lm2, s = Dm / Bm;
  T pre = m / T(kMeMeV) * rl * Z13 / dn;
  if (s > T(0)) {
    T X = s < T(100) ? exp(-s) : T(0);
    Lm1 = log(pre / (X + T(2) * T(kMeMeV) * exp(T(0.5)) * rl * Z13 * (T(1) + xi) / den)) - s;
    Lm2 = log(pre / (X + T(2) * T(kMeMeV) * exp(T(1) / T(3)) * rl * Z13 * (T(1) + xi) / den)) - s;
  } else {
    T X = s > T(-100) ? exp(s) : T(0);
    Lm1 = log(pre / (T(1) + T(2) * T(kMeMeV) * exp(T(0.5)) * rl * Z13 * (T(1) + xi) / den * X));
    Lm2 = log(pre / (T(1) + T(2) * T(kMeMeV) * exp(T(1) / T(3)) * rl * Z13 * (T(1) + xi) / den * X));
  }
  T dm = cpf * (Z + zeta) * (T(1) - v) / v * (T(kMeMeV) / m) * (T(kMeMeV) / m) * (Cm1 * Lm1 + Cm2 * Lm2);
  if (dm < T(0)) dm = T(0);
  return (de + dm) * T(0.1) / energy;
}

// src/Materials.jl:802-832, split for the cooperative evaluation: pair_range
// gives the log of the lower asymmetry bound (false: the DCS vanishes),
// pair_point the Gauss-Legendre term i of the integral over the asymmetry.
template <class T>
DP_HD bool pair_range(T Z, T A, T mass, T K, T q, T* tmin) {
  if (Z <= T(0) || A <= T(0) || mass <= T(0) || K <= T(0) || q <= T(0)) return false;
  if (q <= T(4) * T(kElectronMass)) return false;
  if (q >= K + mass * (T(1) - T(0.75) * T(1.6487212707) * pow(Z, T(1) / T(3)))) return false;
  T gamma = T(1) + K / mass;
  T x0 = T(1) - T(4) * T(kElectronMass) / q, x1 = T(1) - T(6) / (gamma * (gamma - q / mass));
  if (!(x0 > T(0) && x1 > T(0))) return false;
  T ri = T(1) - sqrt(x0) * x1;
  if (ri <= T(0) || ri >= T(1)) return false;
  *tmin = log(ri);
  return true;
}
template <class T>
DP_HD T pair_point(T Z, T A, T mass, T K, T q, T tmin, int i, T scale = T(1)) {
  T r = exp(gl12_t<T>(i, false) * tmin);
  return pair_d2(Z, A, mass, K, q, r, scale) * r * gl12_t<T>(i, true) * tmin;
}
template <class T>
DP_HD T dcs_pair(T Z, T A, T mass, T K, T q, T scale = T(1)) {
  T tmin;
  if (!pair_range(Z, A, mass, K, q, &tmin)) return T(0);
  T I = T(0);
  for (int i = 0; i < 12; ++i) I -= pair_point(Z, A, mass, K, q, tmin, i, scale);
  return I < T(0) ? T(0) : I;
}

// src/Materials.jl:838-926
template <class T>
DP_HD T f2p_allm97(T x, T Q2) {
  const T m02 = T(0.31985), mP2 = T(49.457), mR2 = T(0.15052), Q02 = T(0.52544), L2 = T(0.06527);
  T M = T(0.5) * (T(kProtonMass) + T(kNeutronMass)), M2 = M * M;
  T W2 = M2 + Q2 * (T(1) / x - T(1));
  T t = log(log((Q2 + Q02) / L2) / log(Q02 / L2));
  T xP = (Q2 + mP2) / (Q2 + mP2 + W2 - M2), xR = (Q2 + mR2) / (Q2 + mR2 + W2 - M2);
  T cP = T(0.28067) + (T(0.28067) - T(0.22291)) * (T(1) / (T(1) + pow(t, T(2.1979))) - T(1));
  T aP = T(-0.0808) + (T(-0.0808) + T(0.44812)) * (T(1) / (T(1) + pow(t, T(1.1709))) - T(1));
  T bP = T(0.36292) + T(1.8917) * pow(t, T(1.8439));
  T cR = T(0.80107) + T(0.97307) * pow(t, T(3.4942));
  T aR = T(0.58400) + T(0.37888) * pow(t, T(2.6063));
  T bR = T(0.01147) + T(3.7582) * pow(t, T(0.49338));
  T F2P = cP * exp(aP * log(xP) + bP * log(T(1) - x));
  T F2R = cR * exp(aR * log(xR) + bR * log(T(1) - x));
  return Q2 / (Q2 + m02) * (F2P + F2R);
}
template <class T>
DP_HD T photo_d2(T Z, T A, T ml, T K, T q, T Q2, T scale = T(1)) {
  T cf = T(4) * T(kPi) * T(kAlpha) * T(kAlpha) * T(kHbarC) * T(kHbarC) * scale;
  T M = T(0.5) * (T(kProtonMass) + T(kNeutronMass)), E = K + ml, y = q / E, x = T(0.5) * Q2 / (M * q);
  T F2p = f2p_allm97(x, Q2);
  T sh = T(1);
  if (Z != T(1)) {
    if (x < T(0.0014)) sh = exp(T(-0.1) * log(A));
    else if (x < T(0.04)) sh = exp((T(0.069) * log10(x) + T(0.097)) * log(A));
  }
  T F2A = F2p * sh * (Z + (A - Z) * (T(1) + x * (T(-1.85) + x * (T(2.45) + x * (T(-2.35) + x)))));
  T dds = (T(1) - y + T(0.5) * (T(1) - T(2) * ml * ml / Q2) * (y * y + Q2 / (E * E))) / (Q2 * Q2) -
          T(0.25) / (E * E * Q2);
  return cf * F2A * dds / q;
}
// Split like the pair DCS: photo_range gives log Q2min and the log width.
template <class T>
DP_HD bool photo_range(T Z, T A, T m, T K, T q, T* lmin, T* dx) {
  if (Z <= T(0) || A <= T(0) || m <= T(0) || K <= T(0) || q <= T(0)) return false;
  T M = T(0.5) * (T(kNeutronMass) + T(kProtonMass)), mpi = T(kPionMass);
  if (q <= mpi + T(0.5) * mpi * mpi / M || q >= K + m - T(0.5) * (M + m * m / M)) return false;
  T E = K + m, ml2 = m * m;
  T Q2min = ml2 * (q * q - T(0.5) * ml2) / (E * (E - q));
  T Q2max = T(2) * M * (q - mpi) - mpi * mpi;
  if (Q2max < Q2min || Q2min < T(0)) return false;
  *lmin = log(Q2min);
  *dx = log(Q2max) - *lmin;
  return true;
}
template <class T>
DP_HD T photo_point(T Z, T A, T m, T K, T q, T lmin, T dx, int i, T scale = T(1)) {
  T Q2 = exp(lmin + dx * gl9_t<T>(i, false));
  T v = photo_d2(Z, A, m, K, q, Q2, scale);
  return v > T(0) ? v * (gl9_t<T>(i, true) * dx * Q2) : T(0);
}
template <class T>
DP_HD T dcs_photo(T Z, T A, T m, T K, T q, T scale = T(1)) {
  T lmin, dx;
  if (!photo_range(Z, A, m, K, q, &lmin, &dx)) return T(0);
  T ds = T(0);
  for (int i = 0; i < 9; ++i) ds += photo_point(Z, A, m, K, q, lmin, dx, i, scale);
  return ds < T(0) ? T(0) : ds;
}

// src/Materials.jl:513-528
template <class T>
DP_HD T dcs_ionisation(T Z, T I, T m, T K, T q, T scale = T(1)) {
  T P2 = K * (K + T(2) * m), E = K + m;
  T Wmax = T(2) * T(kElectronMass) * P2 / (m * m + T(kElectronMass) * (T(kElectronMass) + T(2) * E));
  if (q > Wmax) return T(0);
  if (q <= (T(13.6) / T(19.2)) * I) return T(0);
  T E2 = E * E, b2 = P2 / E2;
  return T(2) * T(kPi) * T(kElectronMass) * T(kElectronRadius) * T(kElectronRadius) * Z * scale *
         (T(0.5) / E2 + T(1) / q * (T(1) / q - b2 / Wmax)) / b2;
}

}  // namespace dp

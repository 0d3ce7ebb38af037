// physics_build.cu -- host-side construction of the muon physics tables,
// the product counterpart of create_physics(MUON) without PUMAS dE/dx files:
// src/Physics.jl:280-408 (create_material_table_empirical), :534-599
// (create_physics), src/Materials.jl:360-507 (atomic shells, Fano density
// effect, electronic stopping) and :939-1007 (DCS energy moments).
#include <algorithm>
#include <atomic>
#include <cmath>
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

}  // namespace

// src/Physics.jl:280-408.  Columns per DP_COL_*; Coulomb columns (LB1, LBE,
// MU0, ECUT) are left zero: the scattering tables are not built here.
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
  for (int i = 0; i < n; ++i) {
    double K = E[i], g = 1.0 + K / mass, b = std::sqrt(1.0 - 1.0 / (g * g));
    double p = std::sqrt(K * (K + 2 * mass)), e = K + mass;
    C(DP_COL_FSPIN)[i] = K * (e + mass) / (e * e);
    C(DP_COL_MAGROT)[i] = kLarmor / (b * p);
    C(DP_COL_ECUT)[i] = 0.0;  // mu0 = 0 -> 2 sqrt(0)
  }
}

double host_dcs_moment(int proc, double Z, double A, double I, double mass, double K, double xlo,
                       double xhi, int mode) {
  return dcs_moment(proc, Z, A, I, mass, K, xlo, xhi, mode);
}

}  // namespace dp

// tables.cpp -- oracle restatement of the table builders of src/Physics.jl
// (empirical and dE/dx-file tables, composite/mixture integration) and of the
// dE/dx text parser of src/DEDXLoader.jl.  TEST INFRASTRUCTURE ONLY.
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "oracle.hpp"

namespace orc {

int Physics::index(const std::string& name) const {
  for (size_t i = 0; i < t.size(); ++i)
    if (t[i].name == name) return int(i);
  return -1;
}

double interp_plain(double x, const std::vector<double>& xs, const std::vector<double>& lxs,
                    const std::vector<double>& ys) {
  return interp_fast<double>(x, std::log(x), xs, lxs, ys);
}

// Trapezoid ranges and proper time shared by every builder:
// src/Physics.jl:364-388 (empirical), :183-202/:227-232 (dE/dx), :466-492 (composite).
static void integrate_range(const std::vector<double>& E, const std::vector<double>& S,
                            std::vector<double>& R) {
  size_t n = E.size();
  R.assign(n, 0.0);
  R[0] = E[0] / S[0];
  for (size_t i = 1; i < n; ++i) R[i] = R[i - 1] + (E[i] - E[i - 1]) / ((S[i] + S[i - 1]) / 2);
}
static void integrate_time(const std::vector<double>& E, const std::vector<double>& S,
                           double mass, std::vector<double>& T) {
  size_t n = E.size();
  T.assign(n, 0.0);
  for (size_t i = 1; i < n; ++i) {
    double K = E[i], Kp = E[i - 1];
    double g = 1.0 + K / mass, gp = 1.0 + Kp / mass;
    double b = std::sqrt(1.0 - 1.0 / (g * g)), bp = std::sqrt(1.0 - 1.0 / (gp * gp));
    double gm = (g + gp) / 2, bm = (b + bp) / 2, sm = (S[i] + S[i - 1]) / 2;
    T[i] = T[i - 1] + (K - Kp) / (sm * bm * gm);
  }
}
// src/Physics.jl:243-256 / :392-396 / :505-518 (per-node kinematic columns)
static void finish_kinematics(MaterialTable& t, double mass) {
  size_t n = t.E.size();
  t.fspin.resize(n);
  t.magrot.resize(n);
  t.elastic_cutoff.resize(n);
  for (size_t i = 0; i < n; ++i) {
    double K = t.E[i], g = 1.0 + K / mass, b = std::sqrt(1.0 - 1.0 / (g * g));
    double p = std::sqrt(K * (K + 2 * mass)), e = K + mass;
    t.fspin[i] = K * (e + mass) / (e * e);
    t.magrot[i] = LARMOR_FACTOR / (b * p);
    double mu0 = t.mu0[i];
    t.elastic_cutoff[i] = mu0 < 1e-8 ? 2.0 * std::sqrt(std::max(mu0, 0.0))
                                     : std::acos(std::max(1.0 - 2.0 * mu0, -1.0));
  }
}

// src/Physics.jl:280-408 (create_material_table_empirical)
MaterialTable build_table_empirical(const BaseMaterial& m, double mass,
                                    const std::vector<double>& energies, double cutoff,
                                    double elastic_ratio, bool coulomb) {
  MaterialTable t;
  size_t n = energies.size();
  t.name = m.name;
  t.density = m.density;
  t.I = m.I;
  t.ZoA = m.ZoA;
  t.recipe = m;
  t.E = energies;
  t.logE.resize(n);
  for (size_t i = 0; i < n; ++i) t.logE[i] = std::log(energies[i]);
  t.csda_S.assign(n, 0);
  t.mixed_S.assign(n, 0);
  t.strag.assign(n, 0);
  t.ion.assign(n, 0);
  t.brems.assign(n, 0);
  t.pair.assign(n, 0);
  t.photo.assign(n, 0);
  t.xs.assign(n, 0);
  const double xlow = 1e-6;
#pragma omp parallel for schedule(dynamic)
  for (long ii = 0; ii < long(n); ++ii) {
    size_t i = size_t(ii);
    double K = energies[i];
    double br = 0, pa = 0, ph = 0, hard = 0, cs = 0, st = 0;
    if (K >= 1e-6) {
      for (size_t j = 0; j < m.elements.size(); ++j) {
        const Element& e = m.elements[j];
        double f = m.fractions[j];
        br += f * compute_dcs_integral(BREMS, e.Z, e.A, e.I, mass, K, xlow, 1.0, 1);
        pa += f * compute_dcs_integral(PAIR, e.Z, e.A, e.I, mass, K, xlow, 1.0, 1);
        ph += f * compute_dcs_integral(PHOTO, e.Z, e.A, e.I, mass, K, xlow, 1.0, 1);
        for (int p : {BREMS, PAIR, PHOTO, IONI}) {
          hard += f * compute_dcs_integral(p, e.Z, e.A, e.I, mass, K, cutoff, 1.0, 1);
          cs += f * compute_dcs_integral(p, e.Z, e.A, e.I, mass, K, cutoff, 1.0, 0);
        }
        st += f * compute_dcs_integral(IONI, e.Z, e.A, e.I, mass, K, 0.0, cutoff, 2);
      }
    }
    double el = 0;
#pragma omp critical
    el = electronic_stopping_power(m, mass, K);  // shell cache is not thread safe
    t.ion[i] = el;
    t.brems[i] = br;
    t.pair[i] = pa;
    t.photo[i] = ph;
    t.csda_S[i] = el + br + pa + ph;
    t.mixed_S[i] = std::max(t.csda_S[i] - hard, 1e-20);
    t.strag[i] = st;
    t.xs[i] = cs;
  }
  integrate_range(t.E, t.csda_S, t.csda_R);
  integrate_range(t.E, t.mixed_S, t.mixed_R);
  integrate_time(t.E, t.csda_S, mass, t.csda_T);
  t.lb1.assign(n, 0);
  t.lbe.assign(n, 0);
  t.mu0.assign(n, 0);
  if (coulomb)
    compute_coulomb_tables(m, mass, elastic_ratio, cutoff, t.E, t.csda_R, m.ZoA, m.I, m.density,
                           t.lb1, t.lbe, t.mu0);
  finish_kinematics(t, mass);
  return t;
}

// src/DEDXLoader.jl:54-189 (header scan then 11 numeric columns, MeV cm^2/g)
DedxData load_dedx(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  DedxData d;
  std::string line;
  bool data = false;
  while (std::getline(f, line)) {
    if (!data) {
      auto p = line.find("<Z/A> =");
      if (p != std::string::npos) d.ZoA = std::stod(line.substr(p + 7));
      if (line.find("[MeV]") != std::string::npos && line.find("[MeV/c]") != std::string::npos)
        data = true;
      continue;
    }
    std::istringstream is(line);
    double v[11];
    int k = 0;
    while (k < 11 && (is >> v[k])) ++k;
    if (k < 11) continue;
    d.K.push_back(v[0] * 1e-3);
    d.ion.push_back(v[2] * 1e-4);
    d.brems.push_back(v[3] * 1e-4);
    d.pair.push_back(v[4] * 1e-4);
    d.photo.push_back(v[5] * 1e-4);
    d.S.push_back(v[7] * 1e-4);
    d.R.push_back(v[8] * 10.0);
  }
  return d;
}

// src/Physics.jl:146-273 (create_material_table_from_dedx)
MaterialTable build_table_from_dedx(const DedxData& d, const BaseMaterial& m, double mass,
                                    double cutoff, double elastic_ratio, bool coulomb) {
  MaterialTable t;
  size_t n = d.K.size();
  t.name = m.name;
  t.density = m.density;
  t.I = m.I;
  t.ZoA = d.ZoA;
  t.recipe = m;
  t.E = d.K;
  t.logE.resize(n);
  for (size_t i = 0; i < n; ++i) t.logE[i] = std::log(t.E[i]);
  t.csda_S = d.S;
  t.csda_R = d.R;
  t.ion = d.ion;
  t.brems = d.brems;
  t.pair = d.pair;
  t.photo = d.photo;
  integrate_time(t.E, t.csda_S, mass, t.csda_T);
  t.mixed_S.assign(n, 0);
  t.strag.assign(n, 0);
  t.xs.assign(n, 0);
#pragma omp parallel for schedule(dynamic)
  for (long ii = 0; ii < long(n); ++ii) {
    size_t i = size_t(ii);
    double K = t.E[i], hard = 0, st = 0, cs = 0;
    if (K >= 1e-3) {
      for (size_t j = 0; j < m.elements.size(); ++j) {
        const Element& e = m.elements[j];
        double f = m.fractions[j];
        for (int p : {BREMS, PAIR, PHOTO}) {
          hard += f * compute_dcs_integral(p, e.Z, e.A, e.I, mass, K, cutoff, 1.0, 1);
        }
        hard += f * compute_dcs_integral(IONI, e.Z, e.A, e.I, mass, K, cutoff, 1.0, 1);
        st += f * compute_dcs_integral(IONI, e.Z, e.A, e.I, mass, K, 0.0, cutoff, 2);
        for (int p : {BREMS, PAIR, PHOTO})
          cs += f * compute_dcs_integral(p, e.Z, e.A, e.I, mass, K, cutoff, 1.0, 0);
        cs += f * compute_dcs_integral(IONI, e.Z, e.A, e.I, mass, K, cutoff, 1.0, 0);
      }
    }
    t.mixed_S[i] = std::max(t.csda_S[i] - hard, 1e-20);
    t.strag[i] = st;
    t.xs[i] = cs;
  }
  integrate_range(t.E, t.mixed_S, t.mixed_R);
  t.lb1.assign(n, 0);
  t.lbe.assign(n, 0);
  t.mu0.assign(n, 0);
  if (coulomb)
    compute_coulomb_tables(m, mass, elastic_ratio, cutoff, t.E, t.csda_R, d.ZoA, m.I, m.density,
                           t.lb1, t.lbe, t.mu0);
  finish_kinematics(t, mass);
  return t;
}

// src/Physics.jl:534-599 with the empirical fallback (no dE/dx files).
Physics create_physics(int n_energies, double Kmin, double Kmax,
                       const std::vector<BaseMaterial>& mats, bool coulomb) {
  Physics p;
  std::vector<double> E(n_energies);
  for (int i = 0; i < n_energies; ++i)
    E[i] = Kmin * std::pow(Kmax / Kmin, double(i) / double(n_energies - 1));
  for (const auto& m : mats)
    p.t.push_back(build_table_empirical(m, p.mass, E, p.cutoff, p.elastic_ratio, coulomb));
  return p;
}

// src/Physics.jl:1058-1105 (_build_mixture_table): integrated mixture range and
// proper time on the first table's grid.
MixtureTable build_mixture_table(const Physics& p, const Mixture& mix) {
  MixtureTable mt;
  const MaterialTable& ref = p.t[0];
  size_t n = ref.E.size();
  mt.E = ref.E;
  mt.logE = ref.logE;
  auto stop = [&](bool mixed, double K) {
    double v = 0;
    for (size_t j = 0; j < mix.mats.size(); ++j) {
      const MaterialTable& tb = p.t[mix.mats[j]];
      v += mix.fracs[j] * interp_plain(K, tb.E, tb.logE, mixed ? tb.mixed_S : tb.csda_S);
    }
    return v;
  };
  mt.csda_R.assign(n, 0);
  mt.mixed_R.assign(n, 0);
  mt.csda_T.assign(n, 0);
  double cp = stop(false, mt.E[0]), mp = stop(true, mt.E[0]);
  mt.csda_R[0] = mt.E[0] / cp;
  mt.mixed_R[0] = mt.E[0] / mp;
  for (size_t i = 1; i < n; ++i) {
    double K = mt.E[i], Kp = mt.E[i - 1], dK = K - Kp;
    double c = stop(false, K), m = stop(true, K);
    mt.csda_R[i] = mt.csda_R[i - 1] + dK / ((c + cp) / 2);
    mt.mixed_R[i] = mt.mixed_R[i - 1] + dK / ((m + mp) / 2);
    double g = 1.0 + K / p.mass, gp = 1.0 + Kp / p.mass;
    double b = std::sqrt(1.0 - 1.0 / (g * g)), bp = std::sqrt(1.0 - 1.0 / (gp * gp));
    mt.csda_T[i] = mt.csda_T[i - 1] + dK / (((c + cp) / 2) * ((b + bp) / 2) * ((g + gp) / 2));
    cp = c;
    mp = m;
  }
  return mt;
}

}  // namespace orc

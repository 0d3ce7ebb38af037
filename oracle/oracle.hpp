// oracle.hpp -- FP64 CPU restatement of the DiffPumas.jl hot path.
//
// TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the GPU library:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
// load it.  The product path never calls it.
//
// Every function cites the reference source (paths inside the DiffPumas.jl
// project) it restates.  Gradients are computed with forward-mode dual
// numbers through the same discrete program (the quantity Zygote
// differentiates in the reference), plus central finite differences in tests.
#pragma once
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- constants
// src/Constants.jl:17-92
constexpr double ALPHA_EM = 7.2973525693e-3;
constexpr double HBAR_C = 1.973269804e-16;
constexpr double BOHR_RADIUS = 0.529177210903e-10;
constexpr double MUON_C_TAU = 658.654;
constexpr double ELECTRON_MASS = 0.510998910e-3;
constexpr double ELECTRON_RADIUS = 2.817940285e-15;
constexpr double MUON_MASS = 0.10565839;
constexpr double PROTON_MASS = 0.938272;
constexpr double NEUTRON_MASS = 0.939565;
constexpr double PION_MASS = 0.13957018;
constexpr double AVOGADRO_NUMBER = 6.02214076e23;
constexpr double LARMOR_FACTOR = 0.299792458;
constexpr double DEFAULT_CUTOFF = 5e-2;
constexpr double DEFAULT_ELASTIC_RATIO = 5e-2;
constexpr double STEP_MIN = 1e-7;
constexpr double EHS_PATH_MAX = 1e9;
constexpr double PI = 3.14159265358979323846;
constexpr double EPS64 = 2.220446049250313e-16;  // Julia eps(Float64)
constexpr double PRIMARY_ALTITUDE = 3e4;          // src/Geometry.jl:38

// ---------------------------------------------------------------- dual numbers
// Scalar tangent: value v and derivative d with respect to one seeded input.
struct Dual {
  double v = 0, d = 0;
  Dual() = default;
  Dual(double x) : v(x), d(0) {}
  Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) {
  double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
inline bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
inline Dual log(Dual a) { return {std::log(a.v), a.d / a.v}; }
inline Dual exp(Dual a) {
  double e = std::exp(a.v);
  return {e, e * a.d};
}
inline Dual sqrt(Dual a) {
  double s = std::sqrt(a.v);
  return {s, a.d / (2 * s)};
}
inline Dual abs(Dual a) { return a.v < 0 ? -a : a; }
inline bool isfinite(Dual a) { return std::isfinite(a.v); }
inline double log(double a) { return std::log(a); }
inline double exp(double a) { return std::exp(a); }
inline double sqrt(double a) { return std::sqrt(a); }
inline double abs(double a) { return std::fabs(a); }
inline bool isfinite(double a) { return std::isfinite(a); }
inline double val(double x) { return x; }
inline double val(Dual x) { return x.v; }
inline double der(double) { return 0.0; }
inline double der(Dual x) { return x.d; }
// Julia min/max on reals: the returned operand carries its tangent.
template <class T> inline T jmin(T a, T b) { return (b < a) ? b : a; }
template <class T> inline T jmax(T a, T b) { return (b > a) ? b : a; }

// ---------------------------------------------------------------- materials
// src/Materials.jl:28-127
struct Element {
  std::string name;
  double Z, A, I;
};
struct BaseMaterial {
  std::string name;
  double density, I;
  std::vector<Element> elements;
  std::vector<double> fractions;  // normalised mass fractions
  double ZoA;
};
BaseMaterial make_material(const std::string& name, double density, double I,
                           const std::vector<Element>& els, const std::vector<double>& fr);
const Element& element(const std::string& sym);
BaseMaterial standard_rock();
BaseMaterial air();
BaseMaterial water();

// ---------------------------------------------------------------- tables
// src/Physics.jl:64-102 (MaterialTable)
struct MaterialTable {
  std::string name;
  double density = 0, I = 0, ZoA = 0;
  std::vector<double> E, logE;
  std::vector<double> csda_S, csda_R, csda_T;
  std::vector<double> mixed_S, mixed_R, strag;
  std::vector<double> ion, brems, pair, photo;
  std::vector<double> xs, lb1, lbe, elastic_cutoff, magrot, mu0, fspin;
  BaseMaterial recipe;  // elemental recipe (PhysicsMetadata)
};
struct Physics {
  double mass = MUON_MASS, ctau = MUON_C_TAU;
  double cutoff = DEFAULT_CUTOFF, elastic_ratio = DEFAULT_ELASTIC_RATIO;
  std::vector<MaterialTable> t;
  int index(const std::string& name) const;  // 0-based, -1 if absent
};

// ---------------------------------------------------------------- DCS
double math_dilog(double x);
void gauss_legendre01(int n, double* x, double* w);
double radiation_logarithm(double Z);
double dcs_bremsstrahlung_ssr(double Z, double A, double m, double K, double q);
double dcs_pair_production_ssr(double Z, double A, double m, double K, double q);
double dcs_photonuclear_drss(double Z, double A, double m, double K, double q);
double electronic_dcs(double Z, double I, double m, double K, double q);
double dcs_ionisation_integrate(double Z, double A, double I, double mass, double K,
                                double xlow, double xhigh, int mode);
enum Proc { BREMS = 0, PAIR = 1, PHOTO = 2, IONI = 3 };
double compute_dcs_integral(int proc, double Z, double A, double I, double mass,
                            double K, double xlow, double xhigh, int mode, int npoints = 180);
double electronic_stopping_power(const BaseMaterial& m, double mass, double K);

// ---------------------------------------------------------------- builders
MaterialTable build_table_empirical(const BaseMaterial& m, double mass,
                                    const std::vector<double>& energies,
                                    double cutoff, double elastic_ratio, bool coulomb);
struct DedxData {
  std::vector<double> K, S, R, ion, brems, pair, photo;
  double ZoA = 0;
};
DedxData load_dedx(const std::string& path);
MaterialTable build_table_from_dedx(const DedxData& d, const BaseMaterial& m, double mass,
                                    double cutoff, double elastic_ratio, bool coulomb);
Physics create_physics(int n_energies, double Kmin, double Kmax,
                       const std::vector<BaseMaterial>& mats, bool coulomb);
void compute_coulomb_tables(const BaseMaterial& m, double mass, double elastic_ratio,
                            double cutoff, const std::vector<double>& E,
                            const std::vector<double>& csda_R, double ZoA, double I,
                            double density, std::vector<double>& lb1,
                            std::vector<double>& lbe, std::vector<double>& mu0);

// ---------------------------------------------------------------- mixtures
struct Mixture {
  std::vector<int> mats;        // 0-based material indices
  std::vector<double> fracs;    // normalised
  bool single() const { return mats.size() == 1; }
};
struct MixtureTable {  // src/Physics.jl:996-1002
  std::vector<double> E, logE, csda_R, mixed_R, csda_T;
};
MixtureTable build_mixture_table(const Physics& p, const Mixture& mix);

// ---------------------------------------------------------------- lookups
// src/Physics.jl:660-687 with the rrule of :716-739 (derivative through log x)
template <class T>
T interp_fast(T x, T logx, const std::vector<double>& xs, const std::vector<double>& lxs,
              const std::vector<double>& ys) {
  size_t n = xs.size();
  if (val(x) <= xs[0]) return T(ys[0]);
  if (val(x) >= xs[n - 1]) return T(ys[n - 1]);
  size_t lo = 0, hi = n - 1;
  while (lo < hi - 1) {
    size_t mid = (lo + hi) >> 1;
    if (val(logx) < lxs[mid]) hi = mid; else lo = mid;
  }
  T t = (logx - T(lxs[lo])) / T(lxs[lo + 1] - lxs[lo]);
  return T(ys[lo]) + t * T(ys[lo + 1] - ys[lo]);
}
// src/Physics.jl:833-867 (no rrule: differentiated through t and exp)
template <class T>
T inverse_range(T range, const std::vector<double>& R, const std::vector<double>& E,
                const std::vector<double>& lE) {
  size_t n = R.size();
  if (val(range) <= R[0]) return T(E[0]);
  if (val(range) >= R[n - 1]) return T(E[n - 1]);
  size_t lo = 0, hi = n - 1;
  while (lo < hi - 1) {
    size_t mid = (lo + hi) >> 1;
    if (val(range) < R[mid]) hi = mid; else lo = mid;
  }
  T t = (range - T(R[lo])) / T(R[lo + 1] - R[lo]);
  T logE = T(lE[lo]) + t * T(lE[lo + 1] - lE[lo]);
  return exp(logE);
}
template <class T> T csda_range(const MaterialTable& tb, T E) {
  return interp_fast(E, log(E), tb.E, tb.logE, tb.csda_R);
}
template <class T> T csda_energy(const MaterialTable& tb, T X) {
  return inverse_range(X, tb.csda_R, tb.E, tb.logE);
}
template <class T> T csda_stopping(const MaterialTable& tb, T E) {
  return interp_fast(E, log(E), tb.E, tb.logE, tb.csda_S);
}
double interp_plain(double x, const std::vector<double>& xs, const std::vector<double>& lxs,
                    const std::vector<double>& ys);

// ---------------------------------------------------------------- flux
// src/GaisserFlux.jl:36-133
template <class T> T charge_fraction(T q) {
  const double r = 1.2766;
  if (val(q) < 0) return T(1.0 / (1.0 + r));
  if (val(q) > 0) return T(r / (1.0 + r));
  return T(1.0);
}
double cos_theta_star(double c);
double flux_gaisser(double c, double K, double q);
double flux_gccly(double c, double K, double q);
Dual flux_gccly(double c, Dual K, double q);

// ---------------------------------------------------------------- CSDA geometry
// src/Geometry.jl:47-106 (TwoLayerGeometry without the porous layer)
struct TwoLayer {
  double thickness, primary_altitude;
  int rock, air;  // material indices (0-based)
};
template <class T>
struct FluxResult { T flux; };
// compute_flux_single in deterministic CSDA mode (rng=nothing), with rho as T.
template <class T>
T flux_single_csda(const Physics& p, const TwoLayer& g, T rho, double elevation,
                   double energy, double charge, double energy_threshold,
                   long* steps_out = nullptr);
// Closed-form two-layer CSDA, src/Geometry.jl:1126-1209.
template <class T>
T flux_csda_direct(const Physics& p, int rock, int air, T rho, double thickness,
                   double elevation, double energy, double charge, double primary_altitude);

// ---------------------------------------------------------------- tomography
// examples/diff_flux_cube.jl:85-470 generalised: explicit grid origin/pitch,
// explicit side-exit density.
struct Grid {
  int nx, ny, nz;
  double x0, y0, z0, dx, dy, dz;  // z0 = bottom (detector level)
};
struct Segment {
  int cell;      // 0-based linear index i + nx*(j + ny*k)
  double len;
};
struct Ray {
  double ox, oy, oz;    // start
  double ux, uy, uz;    // unit direction (upward)
  double cos_theta;     // sin(elevation)
};
struct RayTrace {
  std::vector<Segment> seg;
  double z_exit;
};
RayTrace trace_ray(const Grid& g, const Ray& r);
// Density of cell c (or the side-exit remainder when c < 0) with a tangent of
// one on the seeded cell (seed == -2 seeds the side-exit density).
double tomo_node_adjoint(const Physics& p, int rock, int air, const Grid& g, const RayTrace& tr,
                         double cos_theta, const double* rho, double rho_side, double energy,
                         double charge, double H, std::vector<double>& dseg);
template <class T>
T tomo_flux_node(const Physics& p, int rock, int air, const Grid& g,
                 const RayTrace& tr, double cos_theta, const double* rho,
                 double rho_side, int seed, double energy, double charge,
                 double primary_altitude);

}  // namespace orc

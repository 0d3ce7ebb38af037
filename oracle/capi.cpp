// capi.cpp -- flat C entry points of the oracle for the Python test harness
// (ctypes).  TEST INFRASTRUCTURE ONLY: never linked into the product.
#include <algorithm>
#include <cstring>
#include <map>
#include <set>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mc.hpp"
#include "wtomo.hpp"
#include "oracle.hpp"

using namespace orc;

namespace {
struct MatSpec {
  const char* name;
  double density, I;
  int n;
  const double *Z, *A, *Iel, *frac;
};
BaseMaterial to_material(const char* name, double density, double I, int n, const double* Z,
                         const double* A, const double* Iel, const double* frac) {
  std::vector<Element> els;
  std::vector<double> fr;
  for (int i = 0; i < n; ++i) {
    els.push_back({"e", Z[i], A[i], Iel[i]});
    fr.push_back(frac[i]);
  }
  return make_material(name, density, I, els, fr);
}
std::vector<double>* column(MaterialTable& t, int c) {
  switch (c) {
    case 0: return &t.E;
    case 1: return &t.logE;
    case 2: return &t.csda_S;
    case 3: return &t.csda_R;
    case 4: return &t.csda_T;
    case 5: return &t.mixed_S;
    case 6: return &t.mixed_R;
    case 7: return &t.strag;
    case 8: return &t.ion;
    case 9: return &t.brems;
    case 10: return &t.pair;
    case 11: return &t.photo;
    case 12: return &t.xs;
    case 13: return &t.lb1;
    case 14: return &t.lbe;
    case 15: return &t.elastic_cutoff;
    case 16: return &t.magrot;
    case 17: return &t.mu0;
    case 18: return &t.fspin;
  }
  return nullptr;
}
}  // namespace

extern "C" {

// Physics handle: empty, then materials are appended in order.
void* orc_physics_new(double mass, double ctau, double cutoff, double elastic_ratio) {
  Physics* p = new Physics;
  p->mass = mass;
  p->ctau = ctau;
  p->cutoff = cutoff;
  p->elastic_ratio = elastic_ratio;
  return p;
}
void orc_physics_free(void* h) { delete static_cast<Physics*>(h); }

// Empirical table (src/Physics.jl:280) on a log grid of n nodes.
int orc_add_material_empirical(void* h, const char* name, double density, double I, int n_el,
                               const double* Z, const double* A, const double* Iel,
                               const double* frac, int n_energies, double Kmin, double Kmax,
                               int coulomb) {
  Physics* p = static_cast<Physics*>(h);
  std::vector<double> E(n_energies);
  for (int i = 0; i < n_energies; ++i)
    E[i] = Kmin * std::pow(Kmax / Kmin, double(i) / double(n_energies - 1));
  p->t.push_back(build_table_empirical(to_material(name, density, I, n_el, Z, A, Iel, frac),
                                       p->mass, E, p->cutoff, p->elastic_ratio, coulomb != 0));
  return int(p->t.size()) - 1;
}

// dE/dx-file table (src/Physics.jl:146).
int orc_add_material_dedx(void* h, const char* path, const char* name, double density, double I,
                          int n_el, const double* Z, const double* A, const double* Iel,
                          const double* frac, int coulomb) {
  Physics* p = static_cast<Physics*>(h);
  DedxData d = load_dedx(path);
  p->t.push_back(build_table_from_dedx(d, to_material(name, density, I, n_el, Z, A, Iel, frac),
                                       p->mass, p->cutoff, p->elastic_ratio, coulomb != 0));
  return int(p->t.size()) - 1;
}

// Caller-supplied columns (tests overwrite tables with analytic values).
int orc_add_material_columns(void* h, const char* name, double density, double ZoA, int n,
                             const double* const* cols /* 19 columns, see column() */) {
  Physics* p = static_cast<Physics*>(h);
  MaterialTable t;
  t.name = name;
  t.density = density;
  t.ZoA = ZoA;
  for (int c = 0; c < 19; ++c) column(t, c)->assign(cols[c], cols[c] + n);
  p->t.push_back(t);
  return int(p->t.size()) - 1;
}

int orc_table_size(void* h, int mat) { return int(static_cast<Physics*>(h)->t[mat].E.size()); }
int orc_table_column(void* h, int mat, int col, double* out) {
  auto* v = column(static_cast<Physics*>(h)->t[mat], col);
  if (!v) return -1;
  std::copy(v->begin(), v->end(), out);
  return int(v->size());
}

double orc_dcs(int proc, double Z, double A, double I, double m, double K, double q) {
  switch (proc) {
    case BREMS: return dcs_bremsstrahlung_ssr(Z, A, m, K, q);
    case PAIR: return dcs_pair_production_ssr(Z, A, m, K, q);
    case PHOTO: return dcs_photonuclear_drss(Z, A, m, K, q);
    default: return electronic_dcs(Z, I, m, K, q);
  }
}
double orc_dcs_integral(int proc, double Z, double A, double I, double mass, double K,
                        double xlo, double xhi, int mode, int npoints) {
  return compute_dcs_integral(proc, Z, A, I, mass, K, xlo, xhi, mode, npoints);
}
double orc_dilog(double x) { return math_dilog(x); }
double orc_flux_gccly(double c, double K, double q) { return flux_gccly(c, K, q); }
double orc_electronic_stopping(const char* name, double density, double I, int n_el,
                               const double* Z, const double* A, const double* Iel,
                               const double* frac, double mass, double K) {
  return electronic_stopping_power(to_material(name, density, I, n_el, Z, A, Iel, frac), mass, K);
}

// Interpolated property lookups (src/Physics.jl:783-905).
double orc_lookup(void* h, int mat, int col, double K) {
  MaterialTable& t = static_cast<Physics*>(h)->t[mat];
  return interp_plain(K, t.E, t.logE, *column(t, col));
}
double orc_csda_energy(void* h, int mat, double X) {
  MaterialTable& t = static_cast<Physics*>(h)->t[mat];
  return csda_energy<double>(t, X);
}

// One deterministic CSDA history (compute_flux_single with rng = nothing) and
// its density derivative (dual numbers through the discrete program).
void orc_flux_single_csda(void* h, int rock, int air, double thickness, double rho,
                          double elevation, double energy, double charge, double threshold,
                          double primary_altitude, double* flux, double* dflux, long* steps) {
  Physics* p = static_cast<Physics*>(h);
  TwoLayer g{thickness, primary_altitude, rock, air};
  Dual r = flux_single_csda<Dual>(*p, g, Dual(rho, 1.0), elevation, energy, charge, threshold,
                                  steps);
  *flux = r.v;
  *dflux = r.d;
}

// Batch of histories (run_backward_mc CSDA path with recorded samples):
// per-sample contribution w_i*f_i and its density derivative.
void orc_backward_mc_csda(void* h, int rock, int air, double thickness, double rho,
                          double elevation, double threshold, double primary_altitude, long n,
                          const double* E, const double* q, const double* w, double* contrib,
                          double* dcontrib, int nthreads) {
  Physics* p = static_cast<Physics*>(h);
  TwoLayer g{thickness, primary_altitude, rock, air};
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
  for (long i = 0; i < n; ++i) {
    Dual r = flux_single_csda<Dual>(*p, g, Dual(rho, 1.0), elevation, E[i], q[i], threshold,
                                    nullptr);
    contrib[i] = w[i] * r.v;
    dcontrib[i] = w[i] * r.d;
  }
}

void orc_flux_csda_direct(void* h, int rock, int air, double rho, double thickness,
                          double elevation, double energy, double charge, double H,
                          double* flux, double* dflux) {
  Physics* p = static_cast<Physics*>(h);
  Dual r = flux_csda_direct<Dual>(*p, rock, air, Dual(rho, 1.0), thickness, elevation, energy,
                                  charge, H);
  *flux = r.v;
  *dflux = r.d;
}

// Ray trace of one ray: returns segment count (<= cap), cells, lengths, z_exit.
int orc_trace_ray(const int* dims, const double* geom /* x0 y0 z0 dx dy dz */,
                  const double* ray /* ox oy oz ux uy uz cos */, int cap, int* cells,
                  double* lens, double* z_exit) {
  Grid g{dims[0], dims[1], dims[2], geom[0], geom[1], geom[2], geom[3], geom[4], geom[5]};
  Ray r{ray[0], ray[1], ray[2], ray[3], ray[4], ray[5], ray[6]};
  RayTrace tr = trace_ray(g, r);
  int n = std::min<int>(cap, int(tr.seg.size()));
  for (int i = 0; i < n; ++i) {
    cells[i] = tr.seg[i].cell;
    lens[i] = tr.seg[i].len;
  }
  *z_exit = tr.z_exit;
  return int(tr.seg.size());
}

// Tomography forward for many rays: flux_r = (1/N) sum_n 2 w_n f(E_n, q_n).
void orc_tomo_forward(void* h, int rock, int air, const int* dims, const double* geom,
                      const double* rho, double rho_side, double H, long n_rays,
                      const double* rays /* 7 per ray */, int n_nodes, const double* nE,
                      const double* nq, const double* nw, double* flux, int nthreads) {
  Physics* p = static_cast<Physics*>(h);
  Grid g{dims[0], dims[1], dims[2], geom[0], geom[1], geom[2], geom[3], geom[4], geom[5]};
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
  for (long r = 0; r < n_rays; ++r) {
    const double* q = rays + 7 * r;
    Ray ray{q[0], q[1], q[2], q[3], q[4], q[5], q[6]};
    RayTrace tr = trace_ray(g, ray);
    double s = 0;
    for (int k = 0; k < n_nodes; ++k)
      s += 2.0 * nw[k] *
           tomo_flux_node<double>(*p, rock, air, g, tr, q[6], rho, rho_side, -1, nE[k], nq[k], H);
    flux[r] = s / n_nodes;
  }
}

// Forward + reverse-mode adjoint for many rays: flux[r] and
// grad[c] = sum_r cot[r] d flux_r / d rho_c (side-exit remainder at the fixed
// rho_side is not a cell).  Per-thread accumulators, summed in thread order.
void orc_tomo_vjp(void* h, int rock, int air, const int* dims, const double* geom,
                  const double* rho, double rho_side, double H, long n_rays, const double* rays,
                  int n_nodes, const double* nE, const double* nq, const double* nw,
                  const double* cot, double* flux, double* grad, int nthreads) {
  Physics* p = static_cast<Physics*>(h);
  Grid g{dims[0], dims[1], dims[2], geom[0], geom[1], geom[2], geom[3], geom[4], geom[5]};
  long ncell = long(g.nx) * g.ny * g.nz;
  std::vector<std::vector<double>> acc(nthreads > 0 ? nthreads : 1);
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<double>& a = acc[tid];
    a.assign(ncell, 0.0);
    std::vector<double> dseg, tot;
#pragma omp for schedule(dynamic, 4)
    for (long r = 0; r < n_rays; ++r) {
      const double* q = rays + 7 * r;
      Ray ray{q[0], q[1], q[2], q[3], q[4], q[5], q[6]};
      RayTrace tr = trace_ray(g, ray);
      double f = 0;
      tot.assign(tr.seg.size() + 1, 0.0);
      for (int k = 0; k < n_nodes; ++k) {
        double c = 2.0 * nw[k] / n_nodes;
        f += c * tomo_node_adjoint(*p, rock, air, g, tr, q[6], rho, rho_side, nE[k], nq[k], H, dseg);
        for (size_t s = 0; s < dseg.size() && s < tr.seg.size(); ++s) tot[s] += c * dseg[s];
      }
      flux[r] = f;
      for (size_t s = 0; s < tr.seg.size(); ++s) a[tr.seg[s].cell] += cot[r] * tot[s];
    }
  }
  for (long c = 0; c < ncell; ++c) {
    double s = 0;
    for (auto& a : acc)
      if (!a.empty()) s += a[c];
    grad[c] = s;
  }
}

// Stochastic backward MC histories (straggled / mixed / CSDA dual-mode loop).
// rock: n_rock materials with mass fractions; air: material index.  Per
// history i: geometry (thickness, density, elevation, primary altitude) from
// the arrays (index i, or index 0 when the stride flag is 0), final energy
// E[i], charge q[i]; the random stream is (seed, id0 + i).  Outputs the flux
// contribution w[i]*flux, the status bits, the step count and the final energy.
// porous >= 0 adds the shallow porous layer of that material with
// porous_thickness / porous_density (per history when geo_per_history).
void orc_mc_histories(void* h, int n_rock, const int* rock_mats, const double* rock_fracs, int air,
                      long n, const double* thick, const double* dens, const double* elev,
                      const double* H, int geo_per_history, const double* E, const double* q,
                      const double* w, uint64_t seed, uint64_t id0, int straggling, int scattering,
                      double threshold_low, double source_max, double* contrib, int* status,
                      long* steps, double* Efinal, int nthreads, int porous,
                      const double* porous_thickness, const double* porous_density) {
  Physics* p = static_cast<Physics*>(h);
  Mixture rm;
  double tot = 0;
  for (int j = 0; j < n_rock; ++j) tot += rock_fracs[j];
  for (int j = 0; j < n_rock; ++j) {  // MaterialMixture normalises (src/Types.jl:363-368)
    rm.mats.push_back(rock_mats[j]);
    rm.fracs.push_back(rock_fracs[j] / tot);
  }
  Mixture am;
  am.mats.push_back(air);
  am.fracs.push_back(1.0);
  McMedia md;
  md.rock = make_medium(*p, rm);
  md.air = make_medium(*p, am);
  md.krock = prepare_mixed_kernel(*p, rm);
  md.kair = prepare_mixed_kernel(*p, am);
  if (porous >= 0) {
    Mixture pm;
    pm.mats.push_back(porous);
    pm.fracs.push_back(1.0);
    md.has_porous = true;
    md.porous = make_medium(*p, pm);
    md.kporous = prepare_mixed_kernel(*p, pm);
  }
  McOptions o;
  o.straggling = straggling != 0;
  o.scattering = scattering != 0;
  o.energy_threshold_low = threshold_low;
  o.source_energy_max = source_max;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads)
  for (long i = 0; i < n; ++i) {
    long gi = geo_per_history ? i : 0;
    McGeometry geo{thick[gi], dens[gi], elev[gi], H[gi]};
    if (porous >= 0) {
      geo.porous_thickness = porous_thickness[gi];
      geo.porous_density = porous_density[gi];
    }
    Rng g;
    g.seed = seed;
    g.id = id0 + uint64_t(i);
    McState fs;
    double f = stochastic_history(*p, md, geo, E[i], q[i], g, o, &fs);
    contrib[i] = w[i] * f;
    if (status) status[i] = fs.status;
    if (steps) steps[i] = fs.steps;
    if (Efinal) Efinal[i] = fs.E;
  }
}

// Fixed-path MC histories of n_dirs directions (src/Tomography.jl:979-1041).
// Media: n_media mixtures of up to 4 materials (med_mats/med_fracs, 4 per
// medium, med_nm used); segments of direction d are seg_ptr[d]..seg_ptr[d+1]
// (medium index, density, length); samples of direction d are
// smp_ptr[d]..smp_ptr[d+1]; history i uses the Philox stream id0 + i.
// contrib[i] = 2 w_i w flux_gccly, as the reference accumulates it.
void orc_dir_histories(void* h, int n_media, const int* med_nm, const int* med_mats,
                       const double* med_fracs, int rock, double rock_density, int air,
                       double detector_elevation, long n_dirs, const double* cos_theta,
                       const double* remaining_rock, const double* air_distance,
                       const int64_t* seg_ptr, const int* seg_medium, const double* seg_density,
                       const double* seg_length, const int64_t* smp_ptr, const double* E,
                       const double* q, const double* w, uint64_t seed, uint64_t id0,
                       int straggling, double threshold_low, double energy_limit,
                       double* contrib, int* status, long* steps, double* Efinal, int nthreads) {
  Physics* p = static_cast<Physics*>(h);
  DirMedia md;
  for (int k = 0; k < n_media; ++k) {
    Mixture mx;
    double tot = 0;
    for (int j = 0; j < med_nm[k]; ++j) tot += med_fracs[4 * k + j];
    for (int j = 0; j < med_nm[k]; ++j) {  // MaterialMixture normalises (src/Types.jl:363-368)
      mx.mats.push_back(med_mats[4 * k + j]);
      mx.fracs.push_back(med_fracs[4 * k + j] / tot);
    }
    md.med.push_back(make_medium(*p, mx));
    md.kern.push_back(prepare_mixed_kernel(*p, mx));
  }
  md.rock = rock;
  md.air = air;
  md.rock_density = rock_density;
  md.detector_elevation = detector_elevation;
  McOptions o;
  o.straggling = straggling != 0;
  o.scattering = false;
  o.energy_threshold_low = threshold_low;
  o.source_energy_max = energy_limit;
  const long n = long(smp_ptr[n_dirs]);
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads)
  for (long i = 0; i < n; ++i) {
    long d = long(std::upper_bound(smp_ptr, smp_ptr + n_dirs + 1, int64_t(i)) - smp_ptr) - 1;
    DirPath path;
    path.cos_theta = cos_theta[d];
    path.medium = seg_medium + seg_ptr[d];
    path.density = seg_density + seg_ptr[d];
    path.length = seg_length + seg_ptr[d];
    path.n_seg = long(seg_ptr[d + 1] - seg_ptr[d]);
    path.remaining_rock = remaining_rock[d];
    path.air_distance = air_distance[d];
    Rng g;
    g.seed = seed;
    g.id = id0 + uint64_t(i);
    McState fs;
    double f = directional_history(*p, md, path, E[i], q[i], g, o, &fs);
    contrib[i] = 2.0 * w[i] * f;
    if (status) status[i] = fs.status;
    if (steps) steps[i] = fs.steps;
    if (Efinal) Efinal[i] = fs.E;
  }
}

double orc_mc_segment_step(double remaining, double max_step) {
  return mc_segment_step(remaining, max_step);
}

// propagate_mc_uniform_segment of one medium (src/Tomography.jl:876-920).
// state: E, w, distance, grammage, z, u_z in and out; the transport stream is
// (seed, id) or the scripted uniforms; returns the script values consumed.
int orc_dir_segment(void* h, int n_mats, const int* mats, const double* fracs, double* state,
                    double density, double distance, int straggling, double threshold_low,
                    double energy_limit, uint64_t seed, uint64_t id, int n_script,
                    const double* script, int* status) {
  Physics* p = static_cast<Physics*>(h);
  Mixture mx;
  double tot = 0;
  for (int j = 0; j < n_mats; ++j) tot += fracs[j];
  for (int j = 0; j < n_mats; ++j) {
    mx.mats.push_back(mats[j]);
    mx.fracs.push_back(fracs[j] / tot);
  }
  Medium m = make_medium(*p, mx);
  MixedKernel k = prepare_mixed_kernel(*p, mx);
  McState s;
  s.E = state[0];
  s.w = state[1];
  s.dist = state[2];
  s.X = state[3];
  s.z = state[4];
  s.uz = state[5];
  Rng g;
  g.seed = seed;
  g.id = id;
  if (n_script > 0) {
    g.script = script;
    g.n_script = n_script;
  }
  McOptions o;
  o.straggling = straggling != 0;
  o.scattering = false;
  o.energy_threshold_low = threshold_low;
  o.source_energy_max = energy_limit;
  propagate_segment(*p, m, k, s, false, density, distance, -s.uz, 0.0, g, o);
  state[0] = s.E;
  state[1] = s.w;
  state[2] = s.dist;
  state[3] = s.X;
  state[4] = s.z;
  state[5] = s.uz;
  if (status) *status = s.status | (g.overrun ? (1 << 30) : 0);
  return g.pos;
}

// Water-fraction CSDA flux of n_bins paths (compute_directional_flux_csda,
// src/Tomography.jl:667-727) and, when grad is given, d flux / d w of each
// path's cells (directional_flux_and_grad_csda, :736-762) by one tangent per
// distinct cell: grad[j] for segment j holds the derivative with respect to
// its cell at the cell's first segment on the path, 0 at repeats.
// cfg: rock, water, air, porous material indices; dens: rock, water, porous
// densities, porous top thickness; site: detector elevation, primary
// altitude; corr: enabled, kappa_strag, kappa_hard, resid a-d, material
// enabled, linear, quadratic.
void orc_dir_csda(void* h, const int* cfg, const double* dens, const double* site,
                  const double* corr, long n_bins, const double* cos_t, const double* rem,
                  const double* exit_z, const int* valid, const int64_t* seg_ptr,
                  const int* seg_cell, const double* seg_len, long n_cells,
                  const unsigned char* shallow, const double* wf, int n_e, const double* E,
                  const double* q, const double* ew, double* flux, double* grad, int nthreads) {
  Physics* p = static_cast<Physics*>(h);
  WConfig c;
  c.rock = cfg[0];
  c.water = cfg[1];
  c.air = cfg[2];
  c.porous = cfg[3];
  c.rho_rock = dens[0];
  c.rho_water = dens[1];
  c.rho_porous = dens[2];
  c.porous_top = dens[3];
  c.det_elev = site[0];
  c.primary = site[1];
  c.corr = corr[0] != 0.0;
  c.ks = corr[1];
  c.kh = corr[2];
  c.ra = corr[3];
  c.rb = corr[4];
  c.rc = corr[5];
  c.rd = corr[6];
  c.mcorr = corr[7] != 0.0;
  c.lin = corr[8];
  c.quad = corr[9];
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (long b = 0; b < n_bins; ++b) {
    WPath path;
    path.cos_theta = cos_t[b];
    path.remaining_rock = rem[b];
    path.exit_z = exit_z[b];
    path.valid = valid ? valid[b] != 0 : true;
    path.cell = seg_cell + seg_ptr[b];
    path.len = seg_len + seg_ptr[b];
    path.n_seg = long(seg_ptr[b + 1] - seg_ptr[b]);
    flux[b] = dir_flux_csda<double>(*p, c, path, shallow, wf, E, q, ew, n_e);
    if (!grad) continue;
    std::vector<Dual> wd(wf, wf + n_cells);
    for (long k = 0; k < path.n_seg; ++k) {
      double& g = grad[seg_ptr[b] + k];
      g = 0.0;
      bool first = true;
      for (long j = 0; j < k; ++j) first = first && path.cell[j] != path.cell[k];
      if (!first || !path.valid || !(path.cos_theta > 0.0)) continue;
      wd[path.cell[k]].d = 1.0;
      g = dir_flux_csda<Dual>(*p, c, path, shallow, wd.data(), E, q, ew, n_e).d;
      wd[path.cell[k]].d = 0.0;
    }
  }
}

// MixedKernel columns for tests: returns the node count; cols receives
// E, stop, sigma, range, hazard, proper (6 x n, when cap allows) and onset.
int orc_mixed_kernel(void* h, int n_mats, const int* mats, const double* fracs, int cap,
                     double* cols, double* onset) {
  Physics* p = static_cast<Physics*>(h);
  Mixture mx;
  double tot = 0;
  for (int j = 0; j < n_mats; ++j) tot += fracs[j];
  for (int j = 0; j < n_mats; ++j) {
    mx.mats.push_back(mats[j]);
    mx.fracs.push_back(fracs[j] / tot);
  }
  MixedKernel k = prepare_mixed_kernel(*p, mx);
  int n = int(k.E.size());
  if (n <= cap) {
    const std::vector<double>* c[6] = {&k.E, &k.stop, &k.sigma, &k.range, &k.hazard, &k.proper};
    for (int j = 0; j < 6; ++j) std::copy(c[j]->begin(), c[j]->end(), cols + size_t(j) * n);
  }
  *onset = k.onset;
  return n;
}

}  // extern "C"

namespace {
// A MixedKernel from explicit columns (E, stop, sigma, range, hazard, proper;
// n nodes each) and n_el elements of 4 values (Z, A, I, fraction): the
// reference tests build kernels this way (test/test_mixed_kernel.jl).
MixedKernel explicit_kernel(double mass, double ctau, double cutoff, int n, const double* cols,
                            int n_el, const double* el, double onset) {
  MixedKernel c;
  c.mass = mass;
  c.ctau = ctau;
  c.cutoff = cutoff;
  c.onset = onset;
  std::vector<double>* dst[6] = {&c.E, &c.stop, &c.sigma, &c.range, &c.hazard, &c.proper};
  for (int j = 0; j < 6; ++j) dst[j]->assign(cols + size_t(j) * n, cols + size_t(j + 1) * n);
  for (int e = 0; e < n_el; ++e) c.el.push_back({el[4 * e], el[4 * e + 1], el[4 * e + 2], el[4 * e + 3]});
  return c;
}
Rng make_rng(uint64_t seed, uint64_t id, int n_script, const double* script) {
  Rng g;
  g.seed = seed;
  g.id = id;
  if (n_script >= 0) {
    g.script = script;
    g.n_script = n_script;
  }
  return g;
}
}  // namespace

extern "C" {

// One transport_mixed_step on an explicit kernel.  state: E, w, t, x, y, z,
// ux, uy, uz, dist, X (11 values, in and out).  n_script < 0: Philox stream
// (seed, id); else the scripted values.  Returns the status bits; *consumed
// = scripted values used (-1 on overrun).
int orc_mixed_step(double mass, double ctau, double cutoff, int n, const double* cols, int n_el,
                   const double* el, double onset, double* state, double density,
                   double distance, double energy_limit, uint64_t seed, uint64_t id, int n_script,
                   const double* script, int* consumed) {
  MixedKernel c = explicit_kernel(mass, ctau, cutoff, n, cols, n_el, el, onset);
  Rng g = make_rng(seed, id, n_script, script);
  McState s;
  double* f[11] = {&s.E, &s.w, &s.t, &s.x, &s.y, &s.z, &s.ux, &s.uy, &s.uz, &s.dist, &s.X};
  for (int j = 0; j < 11; ++j) *f[j] = state[j];
  transport_mixed_step(c, s, density, distance, g, energy_limit);
  for (int j = 0; j < 11; ++j) state[j] = *f[j];
  if (consumed) *consumed = g.overrun ? -1 : g.pos;
  return s.status;
}

// reverse_del_event on an explicit kernel: out = (energy, weight, process,
// element).  Returns the status bits.
int orc_reverse_del(double mass, double ctau, double cutoff, int n, const double* cols, int n_el,
                    const double* el, double onset, double k, int details, uint64_t seed,
                    uint64_t id, int n_script, const double* script, double* out, int* consumed) {
  MixedKernel c = explicit_kernel(mass, ctau, cutoff, n, cols, n_el, el, onset);
  Rng g = make_rng(seed, id, n_script, script);
  int status = 0;
  DelResult r = reverse_del_event(c, k, g, details != 0, &status);
  out[0] = r.energy;
  out[1] = r.weight;
  out[2] = r.process;
  out[3] = r.element;
  if (consumed) *consumed = g.overrun ? -1 : g.pos;
  return status;
}

// One ray's flux and its density derivative for every cell it touches
// (forward-mode: one dual pass per touched cell, plus the side density).
// Returns the number of touched cells (written up to cap), in first-touch order.
int orc_tomo_ray_grad(void* h, int rock, int air, const int* dims, const double* geom,
                      const double* rho, double rho_side, double H, const double* q, int n_nodes,
                      const double* nE, const double* nq, const double* nw, double* flux,
                      int cap, int* cells, double* grads, double* dside) {
  Physics* p = static_cast<Physics*>(h);
  Grid g{dims[0], dims[1], dims[2], geom[0], geom[1], geom[2], geom[3], geom[4], geom[5]};
  Ray ray{q[0], q[1], q[2], q[3], q[4], q[5], q[6]};
  RayTrace tr = trace_ray(g, ray);
  std::vector<int> uniq;
  std::set<int> seen;
  for (auto& s : tr.seg)
    if (seen.insert(s.cell).second) uniq.push_back(s.cell);
  double f = 0;
  for (int k = 0; k < n_nodes; ++k)
    f += 2.0 * nw[k] *
         tomo_flux_node<double>(*p, rock, air, g, tr, q[6], rho, rho_side, -1, nE[k], nq[k], H);
  *flux = f / n_nodes;
  int m = int(uniq.size());
  for (int u = 0; u <= m; ++u) {
    int seed = u < m ? uniq[u] : -2;
    double d = 0;
    for (int k = 0; k < n_nodes; ++k)
      d += 2.0 * nw[k] *
           tomo_flux_node<Dual>(*p, rock, air, g, tr, q[6], rho, rho_side, seed, nE[k], nq[k], H).d;
    d /= n_nodes;
    if (u < m) {
      if (u < cap) {
        cells[u] = seed;
        grads[u] = d;
      }
    } else {
      *dside = d;
    }
  }
  return m;
}

}  // extern "C"

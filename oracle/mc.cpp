// mc.cpp -- oracle restatement of the stochastic backward Monte Carlo:
// src/MixedTransport.jl (prepared MIXED kernel, adjoint hard events, mixed
// step), src/Straggling.jl (fluctuations, EHS, angles, rotations) and the
// straggled step and dual-mode loop of src/Geometry.jl:148-357, 534-672.
// Random numbers come from the same counter-based Philox streams as the GPU
// kernels (the reference's MersenneTwister stream is not reproducible), so
// histories can be compared one by one.  TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <limits>

#include "mc.hpp"
#include "physics_data.inc"

namespace orc {

// ------------------------------------------------------------ Philox
static inline uint32_t mulhi(uint32_t a, uint32_t b) {
  return uint32_t((uint64_t(a) * uint64_t(b)) >> 32);
}
void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint32_t h0 = mulhi(0xD2511F53u, c[0]), l0 = 0xD2511F53u * c[0];
    uint32_t h1 = mulhi(0xCD9E8D57u, c[2]), l1 = 0xCD9E8D57u * c[2];
    uint32_t n0 = h1 ^ c[1] ^ k0, n2 = h0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = l1;
    c[2] = n2;
    c[3] = l0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}
double Rng::uniform() {
  if (script) {
    if (pos < n_script) return script[pos++];
    overrun = true;
    return std::numeric_limits<double>::quiet_NaN();
  }
  if (used >= 2) {
    uint32_t c[4] = {uint32_t(id), uint32_t(id >> 32), uint32_t(block), uint32_t(block >> 32)};
    philox4x32(c, uint32_t(seed), uint32_t(seed >> 32));
    w[0] = c[0];
    w[1] = c[1];
    w[2] = c[2];
    w[3] = c[3];
    ++block;
    used = 0;
  }
  uint32_t a = w[2 * used], b = w[2 * used + 1];
  ++used;
  return (double(a >> 5) * 67108864.0 + double(b >> 6)) * (1.0 / 9007199254740992.0);
}
double Rng::expo() { return script ? uniform() : -std::log1p(-uniform()); }

// ------------------------------------------------------------ media
Medium make_medium(const Physics& p, const Mixture& mix) {
  Medium m;
  m.mix = mix;
  const MaterialTable& r0 = p.t[mix.mats[0]];
  size_t n = r0.E.size();
  m.E = r0.E;
  m.logE = r0.logE;
  auto wsum = [&](std::vector<double> MaterialTable::*col) {
    std::vector<double> out(n, 0.0);
    for (size_t j = 0; j < mix.mats.size(); ++j)
      for (size_t i = 0; i < n; ++i) out[i] += mix.fracs[j] * (p.t[mix.mats[j]].*col)[i];
    return out;
  };
  if (mix.single()) {
    const MaterialTable& t = p.t[mix.mats[0]];
    m.csda_S = t.csda_S;
    m.mixed_S = t.mixed_S;
    m.strag = t.strag;
    m.xs = t.xs;
    m.mu0 = t.mu0;
    m.fspin = t.fspin;
    m.csda_R = t.csda_R;
    m.mixed_R = t.mixed_R;
    m.csda_T = t.csda_T;
    m.ZoA = t.ZoA;
  } else {
    // src/Physics.jl:1152-1323: weighted sums on the shared grid equal the
    // weighted sums of the interpolated values; ranges from the mixture table
    m.csda_S = wsum(&MaterialTable::csda_S);
    m.mixed_S = wsum(&MaterialTable::mixed_S);
    m.strag = wsum(&MaterialTable::strag);
    m.xs = wsum(&MaterialTable::xs);
    m.mu0 = wsum(&MaterialTable::mu0);
    m.fspin = wsum(&MaterialTable::fspin);
    MixtureTable mt = build_mixture_table(p, mix);
    m.csda_R = mt.csda_R;
    m.mixed_R = mt.mixed_R;
    m.csda_T = mt.csda_T;
    m.ZoA = 0;
    for (size_t j = 0; j < mix.mats.size(); ++j) m.ZoA += mix.fracs[j] * p.t[mix.mats[j]].ZoA;
  }
  return m;
}

static double tl(const Medium& m, const std::vector<double>& col, double x) {
  return interp_plain(x, m.E, m.logE, col);
}
// inverse of a range column (src/Physics.jl:833-867)
static double inv_range(const Medium& m, const std::vector<double>& R, double X) {
  return inverse_range<double>(X, R, m.E, m.logE);
}

// property_transport_path for a single material or mixture (Physics.jl:912, :1220)
static double transport_path(const Physics& p, const Medium& m, double E) {
  if (m.mix.single()) {
    const MaterialTable& t = p.t[m.mix.mats[0]];
    return interp_plain(E, t.E, t.logE, t.lb1);
  }
  double inv = 0.0;
  for (size_t j = 0; j < m.mix.mats.size(); ++j) {
    const MaterialTable& t = p.t[m.mix.mats[j]];
    double lp = interp_plain(E, t.E, t.logE, t.lb1);
    if (lp > 0.0) inv += m.mix.fracs[j] / lp;
  }
  return inv > 0.0 ? 1.0 / inv : 1e9;
}

// compute_ehs_mean_free_path (Straggling.jl:330-360, :1025-1038)
static double ehs_single(const Physics& p, int mat, double K) {
  if (K < 1e-3) return EHS_PATH_MAX;
  const MaterialTable& t = p.t[mat];
  double Lb = interp_plain(K, t.E, t.logE, t.lbe);
  double p2 = K * (K + 2.0 * p.mass);
  if (Lb > 0.0 && Lb < EHS_PATH_MAX * p2) return Lb / p2;
  double tp = interp_plain(K, t.E, t.logE, t.lb1);
  if (tp > 0.0) return std::min(tp / p.elastic_ratio, EHS_PATH_MAX);
  return EHS_PATH_MAX;
}
static double ehs_path(const Physics& p, const Medium& m, double K) {
  if (m.mix.single()) return ehs_single(p, m.mix.mats[0], K);
  double inv = 0.0;
  for (size_t j = 0; j < m.mix.mats.size(); ++j) {
    double lp = ehs_single(p, m.mix.mats[j], K);
    if (lp > 0.0 && lp < EHS_PATH_MAX) inv += m.mix.fracs[j] / lp;
  }
  return inv > 0.0 ? 1.0 / inv : EHS_PATH_MAX;
}

// ------------------------------------------------------------ MixedKernel
// src/MixedTransport.jl:51-97
MixedKernel prepare_mixed_kernel(const Physics& p, const Mixture& mix, int refinement) {
  MixedKernel c;
  c.mass = p.mass;
  c.ctau = p.ctau;
  c.cutoff = p.cutoff;
  double lo = -1e300, hi = 1e300;
  for (int i : mix.mats) {
    lo = std::max(lo, p.t[i].E.front());
    hi = std::min(hi, p.t[i].E.back());
  }
  std::vector<double> grid;
  for (int i : mix.mats)
    for (double e : p.t[i].E)
      if (lo <= e && e <= hi) grid.push_back(e);
  std::sort(grid.begin(), grid.end());
  grid.erase(std::unique(grid.begin(), grid.end()), grid.end());
  for (size_t j = 0; j + 1 < grid.size(); ++j) {
    double a = std::log(grid[j]), b = std::log(grid[j + 1]);
    for (int k = 0; k < refinement; ++k) {
      // Julia range(a, b; length=refinement+1)[k+1] = a + k*(b-a)/refinement
      double x = a + double(k) * (b - a) / double(refinement);
      c.E.push_back(std::exp(x));
    }
  }
  c.E.push_back(hi);
  c.E[0] = lo;
  size_t n = c.E.size();
  auto prop = [&](bool stopping, double k) {
    double v = 0.0;
    for (size_t j = 0; j < mix.mats.size(); ++j) {
      const MaterialTable& t = p.t[mix.mats[j]];
      v += mix.fracs[j] * interp_plain(k, t.E, t.logE, stopping ? t.mixed_S : t.xs);
    }
    return v;
  };
  c.stop.resize(n);
  c.sigma.resize(n);
  for (size_t i = 0; i < n; ++i) {
    c.stop[i] = prop(true, c.E[i]);
    c.sigma[i] = prop(false, c.E[i]);
  }
  c.onset = std::numeric_limits<double>::infinity();
  for (double g : grid) {
    double r = prop(false, g);
    if (r > 0) {
      c.onset = g;
      for (size_t i = 0; i < n; ++i)
        if (c.E[i] < c.onset) c.sigma[i] = r;
      break;
    }
  }
  c.range.assign(n, 0.0);
  c.hazard.assign(n, 0.0);
  c.proper.assign(n, 0.0);
  for (size_t j = 1; j < n; ++j) {
    double a = c.E[j - 1], b = c.E[j], d = b - a;
    c.range[j] = c.range[j - 1] + d / 2 * (1 / c.stop[j - 1] + 1 / c.stop[j]);
    c.hazard[j] = c.hazard[j - 1] + d / 2 * (c.sigma[j - 1] / c.stop[j - 1] + c.sigma[j] / c.stop[j]);
    c.proper[j] = c.proper[j - 1] + d / 2 * p.mass *
                                         (1 / (std::sqrt(a * (a + 2 * p.mass)) * c.stop[j - 1]) +
                                          1 / (std::sqrt(b * (b + 2 * p.mass)) * c.stop[j]));
  }
  for (size_t j = 0; j < mix.mats.size(); ++j) {
    const BaseMaterial& r = p.t[mix.mats[j]].recipe;
    for (size_t k = 0; k < r.elements.size(); ++k)
      c.el.push_back({r.elements[k].Z, r.elements[k].A, r.elements[k].I, mix.fracs[j] * r.fractions[k]});
  }
  return c;
}

// src/MixedTransport.jl:43-49 (searchsortedlast; domain errors become status bits)
static double klookup(double x, const std::vector<double>& xs, const std::vector<double>& ys,
                      int* status) {
  size_t n = xs.size();
  if (x < xs[0]) {
    *status |= ST_DOMAIN_LO;
    return ys[0];
  }
  if (x > xs[n - 1]) {
    *status |= ST_DOMAIN_HI;
    return ys[n - 1];
  }
  size_t i = size_t(std::upper_bound(xs.begin(), xs.end(), x) - xs.begin());  // count <= x
  if (i < 1) i = 1;
  if (i > n - 1) i = n - 1;
  --i;
  double d = xs[i + 1] - xs[i];
  return d == 0 ? ys[i] : ys[i] + (x - xs[i]) / d * (ys[i + 1] - ys[i]);
}

// src/MixedTransport.jl:99-106 components and :111-142 reverse_del_event
static void del_components(const MixedKernel& c, double k, double q, double* v) {
  for (size_t e = 0; e < c.el.size(); ++e) {
    const KEl& x = c.el[e];
    double f = x.fraction * AVOGADRO_NUMBER / (x.A * 0.001) * k;
    v[4 * e + 0] = f * dcs_bremsstrahlung_ssr(x.Z, x.A, c.mass, k, q);
    v[4 * e + 1] = f * dcs_pair_production_ssr(x.Z, x.A, c.mass, k, q);
    v[4 * e + 2] = f * dcs_photonuclear_drss(x.Z, x.A, c.mass, k, q);
    v[4 * e + 3] = f * electronic_dcs(x.Z, x.I, c.mass, k, q);
  }
}
DelResult reverse_del_event(const MixedKernel& c, double k, Rng& rng, bool details, int* status) {
  DelResult r{k, 1.0, 0, -1};
  double sigma = klookup(k, c.E, c.sigma, status);
  if (!(sigma > 0)) {
    *status |= ST_ZERO_RATE;
    return r;
  }
  double pcel = k >= c.onset ? 0.0
                             : -std::log(c.cutoff) /
                                   (-std::log(c.cutoff) + std::log(c.onset / (c.onset - k)));
  if (pcel > 0 && rng.uniform() < pcel) {
    r.weight = 1 / pcel;
    return r;
  }
  const double me = ELECTRON_MASS;
  double xmax = k < 0.5 * (c.mass - me) * (c.mass - me) / me
                    ? std::min(1.0, 2 * me * (k + 2 * c.mass) / ((c.mass + me) * (c.mass + me)))
                    : 1.0;
  double xmin = k >= c.onset * (1 - c.cutoff) ? c.cutoff : 1 - k / c.onset;
  if (!(xmax > xmin)) return r;
  double invnorm = 1 / xmin - 1 / xmax;
  double nu = 1 / (1 / xmin - rng.uniform() * invnorm);
  double rr = 1 - nu, anc = k / rr, pdf = 1 / (invnorm * nu * nu);
  std::vector<double> v(4 * c.el.size());
  del_components(c, anc, anc - k, v.data());
  double total = 0.0;
  for (double x : v) total += x;
  r.energy = anc;
  r.weight = total / (pdf * rr * sigma * (1 - pcel));
  if (details) {
    if (total <= 0) return r;
    double u = rng.uniform() * total;
    for (size_t i = 0; i < v.size(); ++i) {
      u -= v[i];
      if (u <= 0) {
        r.process = int(i % 4) + 1;
        r.element = int(i / 4);
        return r;
      }
    }
    r.process = int((v.size() - 1) % 4) + 1;
    r.element = int((v.size() - 1) / 4);
  }
  return r;
}

// src/MixedTransport.jl:144-200 (transport_mixed_step)
void transport_mixed_step(const MixedKernel& c, McState& s, double density, double distance,
                          Rng& rng, double energy_limit) {
  double k = s.E;
  const double Emax = c.E.back();
  double remaining = distance * density, travelled = 0, proper = 0, weight = s.w;
  double ceiling = energy_limit > 0 ? std::min(energy_limit, Emax) : Emax;
  if (s.E > Emax) {
    s.status |= ST_DOMAIN_HI;
    return;
  }
  bool exhausted = true;
  const double tol = std::nextafter(std::max(1.0, distance * density), 1e300) -
                     std::max(1.0, distance * density);  // eps(max(1, distance*density))
  for (int event = 0; event < 100000; ++event) {
    if (remaining <= tol) {
      exhausted = false;
      break;
    }
    if (k >= ceiling) {
      exhausted = false;
      break;
    }
    double ri = klookup(k, c.E, c.range, &s.status), hi = klookup(k, c.E, c.hazard, &s.status);
    double rtc = std::max(0.0, klookup(ceiling, c.E, c.range, &s.status) - ri);
    double eg = std::min(remaining, rtc);
    double targetr = ri + eg;
    double endpoint = eg == rtc ? ceiling : std::max(k, klookup(targetr, c.range, c.E, &s.status));
    double od = rng.expo();
    double eventh = hi + od;
    bool occurs = eventh < klookup(endpoint, c.E, c.hazard, &s.status);
    double pre = occurs ? std::max(k, klookup(eventh, c.hazard, c.E, &s.status)) : endpoint;
    double dx = occurs ? std::max(0.0, klookup(pre, c.E, c.range, &s.status) - ri) : eg;
    double eps_ri = std::nextafter(std::fabs(ri), 1e300) - std::fabs(ri);
    double eps_k = std::nextafter(std::fabs(k), 1e300) - std::fabs(k);
    double dt;
    if (dx <= 8 * eps_ri || pre - k <= 8 * eps_k)
      dt = dx / density * c.mass / 2 *
           (1 / std::sqrt(k * (k + 2 * c.mass)) + 1 / std::sqrt(pre * (pre + 2 * c.mass)));
    else
      dt = (klookup(pre, c.E, c.proper, &s.status) - klookup(k, c.E, c.proper, &s.status)) / density;
    weight *= klookup(pre, c.E, c.stop, &s.status) / klookup(k, c.E, c.stop, &s.status) *
              std::exp(-dt / c.ctau);
    travelled += dx;
    remaining = std::max(0.0, remaining - dx);
    proper += dt;
    k = pre;
    if (occurs) {
      DelResult d = reverse_del_event(c, k, rng, false, &s.status);
      k = d.energy;
      weight *= d.weight;
      if (!(std::isfinite(weight) && weight >= 0)) s.status |= ST_BAD_WEIGHT;
      if (weight == 0) {
        exhausted = false;
        break;
      }
    } else {
      exhausted = false;
      break;
    }
  }
  if (exhausted) s.status |= ST_EVENT_CAP;
  if (weight > 0 && k >= Emax && remaining > tol && (energy_limit < 0 || k < energy_limit))
    s.status |= ST_DOMAIN_HI;
  double d = travelled / density;
  s.E = k;
  s.w = weight;
  s.t += proper;
  s.dist += d;
  s.X += travelled;
  s.x -= d * s.ux;
  s.y -= d * s.uy;
  s.z -= d * s.uz;
}

// ------------------------------------------------------------ straggling helpers
static double box_muller(Rng& g) {
  double r = std::sqrt(-2.0 * std::log(g.uniform()));
  double phi = 2.0 * PI * g.uniform();
  return r * std::sin(phi);
}
static double truncated_randn(Rng& g) {
  double u = box_muller(g);
  for (int it = 0; it < 1000 && std::fabs(u) > 3.0; ++it) u = box_muller(g);
  return u * 0.9848416472;
}

// src/Straggling.jl:103-173 / :1046-1105 (backward: sgn = -1)
static double fluctuate(const Medium& m, double ki, double dX, double Xtot, Rng& g, double* ratio_out) {
  const double sgn = -1.0;
  double k1 = inv_range(m, m.mixed_R, Xtot - sgn * dX);
  double dk0 = std::fabs(ki - k1), ratio = 1.0;
  if (k1 > 0 && dk0 > 0) {
    double O0 = tl(m, m.strag, ki), O1 = tl(m, m.strag, k1);
    double dk12 = 0.5 * dX * (O0 + O1);
    if (dX / Xtot > 0.05) {
      double de1 = tl(m, m.mixed_S, k1), de0 = tl(m, m.mixed_S, ki);
      dk12 *= 1.0 + sgn * dX / dk0 * (de1 - de0);
    }
    double dk1 = std::sqrt(std::max(dk12, 0.0));
    if (dk0 >= 3.0 * dk1 && dk1 > 0) {
      k1 += truncated_randn(g) * dk1;
    } else if (dk0 >= 1.7320508 * dk1 && dk1 > 0) {
      k1 += 1.7320508 * (1.0 - 2.0 * g.uniform()) * dk1;
    } else if (dk1 > 0) {
      double dk32 = 3.0 * dk12, dk02 = dk0 * dk0;
      double a = 1.0 - (dk32 - dk02) / (dk32 + 3.0 * dk02);
      if (g.uniform() <= a) {
        double b = 0.5 * (dk32 + 3.0 * dk02) / dk0;
        k1 = ki - sgn * b * g.uniform();
        if (k1 < 0) k1 = 0;
      } else {
        k1 = ki;
      }
    }
    ratio = std::fabs(ki - k1) / dk0;
  }
  if (ratio == 0) ratio = 1.0;
  *ratio_out = ratio;
  return std::max(k1, 0.0);
}

// src/Straggling.jl:373-434 / :1284-1334 (backward)
static bool ehs_event(const Physics& p, const Medium& m, double ki, double kf, double dX,
                      double Xtot, double ratio, Rng& g, double* X_ehs, double* k_ehs) {
  const double sgn = -1.0;
  double kmin = std::min(ki, kf), kmax = std::max(ki, kf);
  if (kmin < 0.001) std::swap(kmin, kmax);
  double lb = ehs_path(p, m, kmin);
  if (lb <= 0 || lb >= EHS_PATH_MAX) return false;
  double zeta = g.uniform();
  if (zeta <= 0 || zeta >= 1) return false;
  double X = -std::log(zeta) * lb;
  if (X >= dX) return false;
  double kh = inv_range(m, m.mixed_R, Xtot - sgn * X);
  double k = ki - sgn * ratio * std::fabs(ki - kh);
  if (k <= 0) return false;
  double lbk = ehs_path(p, m, k);
  if (lbk <= 0 || lbk >= EHS_PATH_MAX) return false;
  double r = lbk / lb;
  if (r <= 0 || g.uniform() > 1.0 / r) return false;
  *X_ehs = X;
  *k_ehs = k;
  return true;
}

// src/Straggling.jl:446-517 / :1344-1405
static double scattering_angle(const Physics& p, const Medium& m, double K, Rng& g) {
  double mass = p.mass, p2 = K * (K + 2.0 * mass);
  double mu0 = std::max(tl(m, m.mu0, K), 1e-12);
  double At = m.ZoA > 0 ? 1.0 / m.ZoA : 22.0, Mt = At * NEUTRON_MASS;
  double s = mass * mass + Mt * Mt + 2.0 * (K + mass) * Mt;
  double K0 = (s - (mass + Mt) * (mass + Mt)) / (2.0 * std::sqrt(s));
  double Ecm = K0 + mass, pcm = std::sqrt(std::max(K0 * (K0 + 2.0 * mass), 0.0));
  double El = K + mass, pl = std::sqrt(std::max(p2, 0.0));
  double gCM = (pl > 0 && pcm > 0) ? (El * Ecm + pl * pcm) / (mass * std::sqrt(s)) : 1.0;
  double tau = (pl > 0 && pcm > 0) ? (El * pcm - Ecm * pl) / (pl * pcm) : 0.0;
  double A = mu0 / 4.0, fs = tl(m, m.fspin, K);
  double Apm = A + mu0, Ap1 = A + 1.0, omm = 1.0 - mu0, mu1 = mu0;
  for (int it = 0; it < 100; ++it) {
    double zeta = g.uniform();
    double tmp = Ap1 - zeta * omm;
    if (tmp <= 0) continue;
    double tr = std::min(std::max(Apm * Ap1 / tmp - A, mu0), 1.0);
    if (g.uniform() <= 1.0 - fs * tr) {
      mu1 = tr;
      break;
    }
  }
  double mu;
  if (mu1 > 1e-6) {
    double a = gCM * (tau + 1.0 - 2.0 * mu1);
    double ct = a / std::sqrt(4.0 * mu1 * (1.0 - mu1) + a * a);
    mu = 0.5 * (1.0 - ct);
  } else {
    double d = gCM * (1.0 + tau);
    mu = mu1 / (d * d);
  }
  return std::min(std::max(mu, 0.0), 1.0);
}

// src/Straggling.jl:539-590 / :1204-1253
static double soft_scattering(const Physics& p, const Medium& m, double k0, double k1, double step,
                              double density, Rng& g) {
  if (step <= 0 || density <= 0) return 0.0;
  double lb0 = transport_path(p, m, k0);
  double inv0 = lb0 > 0 ? density / lb0 : 0.0, inv1;
  if (k1 > 0) {
    double lb1 = transport_path(p, m, k1);
    inv1 = lb1 > 0 ? density / lb1 : 0.0;
  } else {
    inv1 = inv0;
  }
  if (inv0 <= 0 && inv1 <= 0) return 0.0;
  double ilb1 = 0.25 * step * (inv0 + inv1);
  if (ilb1 < 1e-12) return 0.0;
  if (ilb1 > 1.0) ilb1 = 1.0;
  for (int it = 0; it < 1000; ++it) {
    double u = g.uniform();
    if (u < 1e-300) continue;
    double mu = -ilb1 * std::log(u);
    if (mu <= 1.0) return std::max(mu, 0.0);
  }
  return ilb1;
}

// src/Straggling.jl:645-710
static void rotate(McState& s, double mu, Rng& g) {
  double ct = 1.0 - 2.0 * mu, st2 = 4.0 * mu * (1.0 - mu);
  if (st2 <= 0) return;
  double st = std::sqrt(st2), d0 = s.ux, d1 = s.uy, d2 = s.uz;
  double ax = std::fabs(d0), ay = std::fabs(d1), az = std::fabs(d2);
  double u0x = 0, u0y = 0, u0z = 0;
  if (ax > ay) {
    if (ax > az) {
      double nrm = 1.0 / std::sqrt(d0 * d0 + d2 * d2);
      u0x = -d2 * nrm;
      u0z = d0 * nrm;
    } else {
      double nrm = 1.0 / std::sqrt(d1 * d1 + d2 * d2);
      u0y = d2 * nrm;
      u0z = -d1 * nrm;
    }
  } else {
    if (ay > az) {
      double nrm = 1.0 / std::sqrt(d0 * d0 + d1 * d1);
      u0x = d1 * nrm;
      u0y = -d0 * nrm;
    } else {
      double nrm = 1.0 / std::sqrt(d1 * d1 + d2 * d2);
      u0y = d2 * nrm;
      u0z = -d1 * nrm;
    }
  }
  double u1x = u0y * d2 - u0z * d1, u1y = u0z * d0 - u0x * d2, u1z = u0x * d1 - u0y * d0;
  double phi = PI * (1.0 - 2.0 * g.uniform());
  double cp = std::cos(phi), sp = std::sin(phi);
  double nx = ct * d0 + st * (cp * u0x + sp * u1x);
  double ny = ct * d1 + st * (cp * u0y + sp * u1y);
  double nz = ct * d2 + st * (cp * u0z + sp * u1z);
  double nrm = std::sqrt(nx * nx + ny * ny + nz * nz);
  if (nrm > 0) {
    nx /= nrm;
    ny /= nrm;
    nz /= nrm;
  }
  s.ux = nx;
  s.uy = ny;
  s.uz = nz;
}

// src/Straggling.jl:726-729 (1-based index of the RMS radius table)
static double rms_radius(double Z) {
  int iZ = std::min(std::max(int(std::lround(Z)), 1), 120);
  return DPDATA_NUCLEAR_RMS_RADII_FM[iZ - 1] * 1e-15;
}

// src/Straggling.jl:746-822
static double polar_brems(double m, double ki, double kf, double Z, Rng& g) {
  double E = ki + m, nu = ki - kf;
  if (nu <= 0 || E <= m) return 0.0;
  double y = nu / E, tmp = 0.5 * m * nu / (E * (E - nu)), mu0 = tmp * tmp;
  double c1 = (2.0 * (1.0 - y) + y * y) * mu0, c2 = 4.0 * (1.0 - y) * mu0 * mu0;
  double RN = rms_radius(Z), t2 = m * RN / HBAR_C, muni = t2 * t2 / 6.0;
  if (std::sqrt(mu0) - mu0 < 0) return 0.0;
  double q0 = muni, r0 = mu0, qr0 = q0 * r0, den0 = r0 + qr0;
  if (den0 <= 0 || (1.0 + qr0) <= 0) return 0.0;
  double x0 = (1.0 + 2.0 * qr0) * std::log((1.0 + qr0) / den0) - (1.0 - r0) * (1.0 + 2.0 * q0) / (1.0 + q0);
  if (x0 <= 0) return 0.0;
  for (int it = 0; it < 100; ++it) {
    double r0r = g.uniform(), r1 = g.uniform();
    double mu = r0r * mu0 / (mu0 + 1.0 - r0r);
    double mus = mu0 + mu, mu2 = mus * mus, d1 = 1.0 / mu2, d2 = d1 * d1;
    double score = r1 * c1 * d1, pdf = c1 * d1 - mu * c2 * d2;
    if (score > pdf) continue;
    double l2 = mu2 / (mu0 * mu0), q = muni * l2, r = mu0 * l2, qr = q * r;
    if (qr > 1e5) continue;
    double den = r + qr;
    if (den <= 0 || (1.0 + qr) <= 0) continue;
    double x = (1.0 + 2.0 * qr) * std::log((1.0 + qr) / den) - (1.0 - r) * (1.0 + 2.0 * q) / (1.0 + q);
    pdf *= x / x0;
    if (score <= pdf) return mu;
  }
  return 0.0;
}
// src/Straggling.jl:834-882
static double polar_photo(double ml, double ki, double kf, Rng& g) {
  double M = 0.5 * (PROTON_MASS + NEUTRON_MASS), q = ki - kf, E = ki + ml, ml2 = ml * ml;
  double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
  double Q2max = 2.0 * M * (q - PION_MASS) - PION_MASS * PION_MASS;
  if (Q2max < Q2min || Q2min < 0) return 0.0;
  double rQ2 = std::log(Q2max) - std::log(Q2min);
  double Q2 = Q2min * std::exp(rQ2 * g.uniform());
  double p = std::sqrt(ki * (ki + 2.0 * ml)), E1 = E - q, er = ml / E1;
  double p1 = E1 * std::sqrt(std::max((1.0 + er) * (1.0 - er), 0.0)), p2 = p * p1;
  if (p2 <= 0) return 0.0;
  double tv = p2 + ml2 - E * E1;
  if (std::fabs(tv) <= 3.0 * EPS64 * p2) tv = 0.0;
  double mu = 0.5 * tv / p2 + 0.25 / p2 * Q2;
  return std::min(std::max(mu, 0.0), 1.0);
}
// src/Straggling.jl:893-914
static double polar_ioni(double m, double ki, double kf) {
  double nu = ki - kf, p2 = ki * (ki + 2.0 * m), E = ki + m;
  double den = std::sqrt(p2 * (p2 + nu * nu - 2.0 * nu * E));
  if (den <= 0) return 0.0;
  double c = (p2 - nu * (E + ELECTRON_MASS)) / den;
  return 0.5 * (1.0 - c);
}

// src/Geometry.jl:148-357 (transport_backward_step_full, mode :straggled)
void straggled_step(const Physics& p, const Medium& m, const MixedKernel& kern, McState& s,
                    double density, double step, Rng& g, bool scattering, double energy_limit) {
  double ki = s.E, mass = p.mass, dX = step * density;
  double Xi = tl(m, m.mixed_R, ki);
  double kf = ki, ratio = 1.0;
  if (ki > 0.001) {
    kf = fluctuate(m, ki, dX, Xi, g, &ratio);
    kf = std::max(kf, ki);
  } else {
    kf = inv_range(m, m.mixed_R, Xi + dX);
  }
  if (energy_limit > 0 && kf >= energy_limit) {
    double dk = std::fabs(ki - kf);
    if (dk > 0) {
      dX = dX * (std::fabs(energy_limit - ki) / dk);
      kf = energy_limit;
    }
  }
  bool del = false, ehs = false;
  double X_del = std::numeric_limits<double>::infinity(), k_del = 0, X_ehs = X_del, k_ehs = 0;
  double rate = std::max(klookup(ki, kern.E, kern.sigma, &s.status), klookup(kf, kern.E, kern.sigma, &s.status));
  if (rate > 0) {
    double cand = g.expo() / rate;
    if (cand < dX) {
      double kh = inv_range(m, m.mixed_R, Xi + cand);
      double pre = ki + ratio * std::fabs(kh - ki);
      if (pre > 0 && g.uniform() <= klookup(pre, kern.E, kern.sigma, &s.status) / rate) {
        del = true;
        X_del = cand;
        k_del = pre;
      }
    }
  }
  if (scattering) {
    double X, k;
    if (ehs_event(p, m, ki, kf, dX, Xi, ratio, g, &X, &k) && k > 0) {
      ehs = true;
      X_ehs = X;
      k_ehs = k;
    }
  }
  if (del && ehs) {
    if (X_del <= X_ehs) ehs = false;
    else del = false;
  }
  double dw = 1.0, ckf = kf;
  int proc = 0, elem = -1;
  if (del) {
    ckf = k_del;
    DelResult d = reverse_del_event(kern, k_del, g, true, &s.status);
    kf = d.energy;
    dw = d.weight;
    proc = d.process;
    elem = d.element;
    dX = X_del;
  }
  if (ehs) {
    kf = k_ehs;
    ckf = k_ehs;
    dX = X_ehs;
  }
  double astep = dX / density;
  // the position moves along the incoming direction; deflections apply after
  double ox = s.ux, oy = s.uy, oz = s.uz;
  if (scattering) {
    if (del && proc > 0) {
      const KEl& e = kern.el[elem];
      double mu = proc == 1 || proc == 2 ? polar_brems(mass, kf, ckf, e.Z, g)
                  : proc == 3            ? polar_photo(mass, kf, ckf, g)
                                         : polar_ioni(mass, kf, ckf);
      if (mu > 0) rotate(s, mu, g);
    }
    if (ehs) {
      double mu = scattering_angle(p, m, k_ehs, g);
      if (mu > 0) rotate(s, mu, g);
    }
    double mu = soft_scattering(p, m, ki, ckf, astep, density, g);
    if (mu > 0) rotate(s, mu, g);
  }
  double pt = astep * mass / 2 * (1.0 / std::sqrt(ki * (ki + 2 * mass)) + 1.0 / std::sqrt(ckf * (ckf + 2 * mass)));
  s.x -= astep * ox;
  s.y -= astep * oy;
  s.z -= astep * oz;
  double wf = tl(m, m.mixed_S, ckf) / tl(m, m.mixed_S, ki);
  s.w = s.w * wf * std::exp(-pt / p.ctau) * dw;
  s.E = kf;
  s.t += pt;
  s.dist += astep;
  s.X += dX;
}

// src/Geometry.jl:424-457 (deterministic CSDA step on a medium)
static void csda_step_medium(const Physics& p, const Medium& m, McState& s, double density,
                             double step) {
  double ki = s.E, dX = step * density;
  double kf = inv_range(m, m.csda_R, tl(m, m.csda_R, ki) + dX);
  double g = (1.0 + ki / p.mass + 1.0 + kf / p.mass) / 2.0;
  double b = std::sqrt(std::max(1.0 - 1.0 / (g * g), 1e-12));
  double dt = step / (b * g);
  s.x -= step * s.ux;
  s.y -= step * s.uy;
  s.z -= step * s.uz;
  s.w = s.w * (tl(m, m.csda_S, kf) / tl(m, m.csda_S, ki)) * std::exp(-dt / p.ctau);
  s.t += dt;
  s.E = kf;
  s.dist += step;
  s.X += dX;
}

// src/Geometry.jl:534-672 with rng (dual-mode loop) and the acceptance of
// :694-757.  Returns the flux contribution (without the sampling weight).
double stochastic_history(const Physics& p, const McMedia& md, const McGeometry& geo, double E0,
                          double q, Rng& g, const McOptions& o, McState* final_state) {
  double theta = (90.0 - geo.elevation) * PI / 180.0;
  McState s;
  s.E = E0;
  s.ux = -std::sin(theta);
  s.uy = 0.0;
  s.uz = -std::cos(theta);
  const double eps = EPS64, H = geo.primary_altitude, low = o.energy_threshold_low;
  const double thr = o.source_energy_max;
  long steps = 0;
  for (int outer = 0; outer < 1000 && s.E < thr - eps; ++outer) {
    if (s.z < 0 || s.z >= H - eps) break;
    if (s.w <= 0 || !std::isfinite(s.w)) break;
    bool strag, mixed, scat;
    double limit;
    if (s.E < low - eps) {
      strag = o.straggling;
      mixed = false;
      scat = o.scattering;
      limit = std::min(low, thr);
    } else {
      strag = false;
      mixed = o.straggling;
      scat = false;
      limit = thr;
    }
    for (int inner = 0; inner < 50000; ++inner) {
      if (s.z < 0 || s.z >= H - eps) break;
      if (s.E >= limit - eps) break;
      if (s.w <= 0 || !std::isfinite(s.w)) break;
      double uz = -s.uz;
      bool in_air = s.z >= geo.thickness;
      // the porous top layer z in [thickness - porous_thickness, thickness)
      // (src/Geometry.jl:617-635)
      const bool has_p = md.has_porous && geo.porous_thickness > 0;
      const double pz = has_p ? geo.thickness - geo.porous_thickness : geo.thickness;
      const bool in_p = !in_air && has_p && s.z >= pz;
      const Medium& m = in_air ? md.air : in_p ? md.porous : md.rock;
      const MixedKernel& k = in_air ? md.kair : in_p ? md.kporous : md.krock;
      double dens, tob;
      if (!in_air) {
        dens = in_p ? geo.porous_density : geo.density;
        const double next = has_p && s.z < pz ? pz : geo.thickness;
        const double prev = has_p && s.z >= pz ? pz : 0.0;
        tob = uz > eps ? (next - s.z) / uz : uz < -eps ? (prev - s.z) / uz : 1000.0;
      } else {
        dens = 1.205 * std::exp(-s.z / 12e3);
        tob = uz > eps ? (H - s.z) / uz : uz < -eps ? (geo.thickness - s.z) / uz : 1000.0;
      }
      // src/Geometry.jl:461-476
      double Xi = tl(m, m.csda_R, s.E);
      double lim = 0.01 * Xi / std::max(dens, 1e-6);
      if (scat) {
        double lb1 = transport_path(p, m, s.E);
        if (lb1 > 0 && dens > 0) lim = std::min(lim, 0.01 * lb1 / dens);
      }
      if (in_air) lim = std::min(lim, 0.05 * 12e3 / std::max(std::fabs(uz), 0.05));
      double step = std::min(tob + 1e-7, lim);
      step = std::min(std::max(step, STEP_MIN), 1000.0);
      if (strag) straggled_step(p, m, k, s, dens, step, g, scat, limit);
      else if (mixed) transport_mixed_step(k, s, dens, step, g, limit);
      else csda_step_medium(p, m, s, dens, step);
      if (++steps > 2000000) s.status |= ST_STEP_CAP;
      if (s.status & ST_FATAL) break;
    }
    if (s.status & ST_FATAL) break;
  }
  s.steps = steps;
  if (final_state) *final_state = s;
  if (s.status & ST_FATAL) return 0.0;
  if (s.z >= H - 1.0 && s.E < thr) {
    double c = std::min(std::max(-s.uz, 0.0), 1.0);
    if (c <= 0) return 0.0;
    return s.w * flux_gccly(c, s.E, q);
  }
  return 0.0;
}

// propagate_mc_uniform_segment / propagate_mc_air_segment
// (src/Tomography.jl:876-969): consume `distance` metres of one medium with
// the segment step rule of :873-874; air takes its density at the current
// altitude above the detector.
double mc_segment_step(double remaining, double max_step) {
  return std::min(remaining, std::max(1e-6, std::min(remaining + 1e-7, max_step)));
}

void propagate_segment(const Physics& p, const Medium& m, const MixedKernel& k, McState& s,
                       bool air, double density, double distance, double cos_theta,
                       double detector_elevation, Rng& g, const McOptions& o) {
  const double eps = EPS64, elimit = o.source_energy_max, low = o.energy_threshold_low;
  double remaining = distance;
  while (remaining > 1e-8 && s.E < elimit - eps) {
    if (s.w <= 0 || !std::isfinite(s.w)) break;
    const double cur = s.E < low - eps ? std::min(low, elimit) : elimit;
    const double rho = air ? 1.205 * std::exp(-(detector_elevation + s.z) / 12e3) : density;
    double mx = 0.01 * tl(m, m.csda_R, s.E) / std::max(rho, air ? 1e-8 : 1e-6);
    if (air) mx = std::min(mx, 0.05 * 12e3 / std::max(cos_theta, 0.05));
    const double step = mc_segment_step(remaining, mx);
    const double d0 = s.dist, E0 = s.E;
    if (s.E < low - eps) {
      if (o.straggling) straggled_step(p, m, k, s, rho, step, g, false, cur);
      else csda_step_medium(p, m, s, rho, step);
    } else {
      if (o.straggling) transport_mixed_step(k, s, rho, step, g, cur);
      else csda_step_medium(p, m, s, rho, step);
    }
    if (++s.steps > 2000000) s.status |= ST_STEP_CAP;
    if (s.status & ST_FATAL) break;
    const double actual = s.dist - d0;
    if (s.w <= 0 || !std::isfinite(s.w)) break;
    // a sub-ulp displacement that reached the mode boundary is progress
    if (actual <= 0 && E0 < cur && cur < elimit && s.E >= cur) continue;
    if (!(actual > 0)) {
      if (s.E >= elimit) break;
      s.status |= ST_NO_PROGRESS;  // the reference raises an error
      break;
    }
    remaining = std::max(0.0, remaining - actual);
  }
}

// compute_directional_flux_mc, one sample (src/Tomography.jl:1009-1034).
double directional_history(const Physics& p, const DirMedia& md, const DirPath& path, double E0,
                           double q, Rng& g, const McOptions& o, McState* final_state) {
  McState s;
  s.E = E0;
  s.ux = s.uy = 0.0;
  s.uz = -path.cos_theta;  // initial_state: direction -dir (src/Tomography.jl:863-869)
  auto ok = [&] { return s.w > 0.0 && std::isfinite(s.w) && !(s.status & (ST_FATAL | ST_NO_PROGRESS)); };
  for (long j = 0; j < path.n_seg; ++j) {
    const int k = path.medium[j];
    propagate_segment(p, md.med[k], md.kern[k], s, false, path.density[j], path.length[j],
                      path.cos_theta, md.detector_elevation, g, o);
    if (!ok()) break;
  }
  if (ok() && path.remaining_rock > 1e-8)
    propagate_segment(p, md.med[md.rock], md.kern[md.rock], s, false, md.rock_density,
                      path.remaining_rock, path.cos_theta, md.detector_elevation, g, o);
  if (ok())
    propagate_segment(p, md.med[md.air], md.kern[md.air], s, true, 0.0, path.air_distance,
                      path.cos_theta, md.detector_elevation, g, o);
  if (final_state) *final_state = s;
  if (s.status & (ST_FATAL | ST_NO_PROGRESS)) return 0.0;
  if (s.w > 0.0 && std::isfinite(s.w) && s.E < o.source_energy_max)
    return s.w * flux_gccly(path.cos_theta, s.E, q);
  return 0.0;
}

}  // namespace orc

// mc.hpp -- oracle types for the stochastic backward Monte Carlo (mc.cpp).
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include "oracle.hpp"

namespace orc {

// History status bits (reference throw sites and loop caps become flags)
enum : int {
  ST_STEP_CAP = 1,     // total step cap
  ST_EVENT_CAP = 4,    // src/MixedTransport.jl:157,193 (100000 hard events)
  ST_DOMAIN_HI = 8,    // src/MixedTransport.jl:45,155,196
  ST_DOMAIN_LO = 16,   // src/MixedTransport.jl:44
  ST_ZERO_RATE = 32,   // src/MixedTransport.jl:113
  ST_BAD_WEIGHT = 64,  // src/MixedTransport.jl:186
  ST_FATAL = ST_STEP_CAP | ST_EVENT_CAP | ST_DOMAIN_HI | ST_DOMAIN_LO | ST_ZERO_RATE | ST_BAD_WEIGHT,
};

void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1);

// Sequential uniforms of history `id`: Philox4x32-10 keyed by the seed, counter
// (id, block); two 32-bit words per double.  Block 0 holds the history's
// energy/charge draws, blocks 1-2 its drawn geometry; transport starts at
// block 3.
struct Rng {
  uint64_t seed = 0, id = 0, block = 3;
  uint32_t w[4] = {0, 0, 0, 0};
  int used = 2;
  // Optional scripted stream (tests): uniform() and expo() both pop the next
  // value, as the reference tests' scripted generators do; past the end they
  // return NaN and set `overrun`.
  const double* script = nullptr;
  int n_script = 0, pos = 0;
  bool overrun = false;
  double uniform();
  double expo();  // -log(1 - U)
};

struct McState {
  double E = 0, w = 1, t = 0, x = 0, y = 0, z = 0, ux = 0, uy = 0, uz = -1;
  double dist = 0, X = 0;  // path length (m) and grammage (kg/m^2)
  int status = 0;
  long steps = 0;
};

// A propagation medium: one material or a runtime mixture on the shared grid.
struct Medium {
  Mixture mix;
  std::vector<double> E, logE, csda_S, mixed_S, strag, xs, mu0, fspin, csda_R, mixed_R, csda_T;
  double ZoA = 0;
};
Medium make_medium(const Physics& p, const Mixture& mix);

struct KEl {
  double Z, A, I, fraction;
};
struct MixedKernel {  // src/MixedTransport.jl:15-29
  double mass, ctau, cutoff, onset;
  std::vector<double> E, stop, sigma, range, hazard, proper;
  std::vector<KEl> el;
};
MixedKernel prepare_mixed_kernel(const Physics& p, const Mixture& mix, int refinement = 8);

struct DelResult {
  double energy, weight;
  int process, element;  // process 0: null CEL event
};
DelResult reverse_del_event(const MixedKernel& c, double k, Rng& rng, bool details, int* status);
void transport_mixed_step(const MixedKernel& c, McState& s, double density, double distance,
                          Rng& rng, double energy_limit);
void straggled_step(const Physics& p, const Medium& m, const MixedKernel& kern, McState& s,
                    double density, double step, Rng& g, bool scattering, double energy_limit);

struct McMedia {
  Medium rock, air;
  MixedKernel krock, kair;
  // shallow porous layer of TwoLayerGeometry (src/Geometry.jl:47-72): a
  // single material
  bool has_porous = false;
  Medium porous;
  MixedKernel kporous;
};
struct McGeometry {
  double thickness, density, elevation, primary_altitude;
  double porous_thickness = 0, porous_density = 0;  // the top of the rock column
};
struct McOptions {
  bool straggling = true, scattering = true;
  double energy_threshold_low = 100.0, source_energy_max = 1e9;
};
double stochastic_history(const Physics& p, const McMedia& md, const McGeometry& geo, double E0,
                          double q, Rng& g, const McOptions& o, McState* final_state);

// Fixed-path MC of one direction (src/Tomography.jl:826-1041): the media a
// path's segments use, the rock beyond them and the air above.
enum : int { ST_NO_PROGRESS = 256 };  // src/Tomography.jl:916,965
struct DirMedia {
  std::vector<Medium> med;
  std::vector<MixedKernel> kern;
  int rock = 0, air = 0;
  double rock_density = 0, detector_elevation = 0;
};
struct DirPath {
  double cos_theta = 1;
  const int* medium = nullptr;      // per segment
  const double* density = nullptr;  // per segment
  const double* length = nullptr;   // per segment
  long n_seg = 0;
  double remaining_rock = 0, air_distance = 0;
};
// _mc_segment_step (src/Tomography.jl:873-874).
double mc_segment_step(double remaining, double max_step);
// propagate_mc_uniform_segment (air = false) or propagate_mc_air_segment.
void propagate_segment(const Physics& p, const Medium& m, const MixedKernel& k, McState& s,
                       bool air, double density, double distance, double cos_theta,
                       double detector_elevation, Rng& g, const McOptions& o);
// One history of compute_directional_flux_mc; returns w * flux_gccly (the
// caller applies 2 * sample weight).  o.source_energy_max is the energy
// limit min(1e9, last table energy).
double directional_history(const Physics& p, const DirMedia& md, const DirPath& path, double E0,
                           double q, Rng& g, const McOptions& o, McState* final_state);

}  // namespace orc

// wtomo.hpp -- oracle types of the water-fraction CSDA forward model
// (src/Tomography.jl:171-820).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "oracle.hpp"

namespace orc {

// MaterialConfig + SiteConfig + the CSDA correction settings
// (src/Tomography.jl:136-201); material indices 0-based, porous < 0: none.
struct WConfig {
  int rock = 0, water = 2, air = 1, porous = -1;
  double rho_rock = 2650, rho_water = 1000, rho_porous = 0, porous_top = 0;
  double det_elev = 0, primary = 3e4;
  bool corr = false;
  double ks = 0, kh = 0, ra = 0, rb = 0, rc = 0, rd = 0;
  bool mcorr = false;
  double lin = 0, quad = 0;
};
// A DirectionalPath (src/Tomography.jl:214-223): cells 0-based.
struct WPath {
  double cos_theta = 1, remaining_rock = 0, exit_z = 0;
  bool valid = true;
  const int* cell = nullptr;
  const double* len = nullptr;
  long n_seg = 0;
};
template <class T>
T dir_flux_csda(const Physics& p, const WConfig& c, const WPath& path, const unsigned char* shallow,
                const T* w, const double* E, const double* q, const double* ew, int n_e);
double spectral_index(double E, double cos_t);

}  // namespace orc

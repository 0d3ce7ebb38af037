// coulomb.cpp -- oracle restatement of src/Coulomb.jl (Coulomb scattering
// tables: transport path, elastic path, screening).  TEST INFRASTRUCTURE ONLY.
#include <stdexcept>

#include "oracle.hpp"

namespace orc {

void compute_coulomb_tables(const BaseMaterial&, double, double, double,
                            const std::vector<double>&, const std::vector<double>&, double,
                            double, double, std::vector<double>&, std::vector<double>&,
                            std::vector<double>&) {
  throw std::runtime_error("Coulomb tables are not restated yet");
}

}  // namespace orc

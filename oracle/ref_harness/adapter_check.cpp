// Compile check — TEST INFRASTRUCTURE ONLY: the reference's own Simulation
// (include/simulation.h) instantiated with the GB300 policies of
// include/gb300_policies.h through include/gb300_config_types.h, the
// replacement of the reference's configTypes.h.  Compiled (syntax only) by
// oracle/ref_build.py's check_adapters() against the reference's headers.
#include <fstream>
#include <iterator>

#include "gb300_config_types.h"

template class Gb300Movement<config::Simulation_t>;
template class Gb300Infection<config::Simulation_t>;
template class Gb300Testing<config::Simulation_t>;
template class Gb300Closure<config::Simulation_t>;

// runSimulation and runForDay call every policy member (simulation.h:899-956)
void gb300_adapter_instantiate(const cxxopts::ParseResult& result) {
    cxxopts::Options options("check", "");
    config::Simulation_t::addProgramParameters(options);
    config::Simulation_t s{result};
    s.runSimulation();
}

// C entry points over the GPU calculator plugin, for callers without C++
// (ctypes, cgo, a test driver): they hold one calculator with its state,
// occupant lists and run manager, built through the factories
// make_GpuCanonicalCalculator / make_GpuSemiGrandCanonicalCalculator and
// driven only through the BaseMonteCalculator / BaseMontePotential
// interface. Errors come back as -1 with the message in
// cem_plugin_last_error.
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "cem.h"
#include "casm/clexmonte/monte_calculator/BaseMonteCalculator.hh"

extern "C" CASM::clexmonte::BaseMonteCalculator *make_GpuCanonicalCalculator();
extern "C" CASM::clexmonte::BaseMonteCalculator *make_GpuSemiGrandCanonicalCalculator();

namespace {

using namespace CASM;
using namespace CASM::clexmonte;

thread_local std::string g_err;

struct PluginCalc {
  std::unique_ptr<BaseMonteCalculator> calc;
  state_type state;
  monte::OccLocation occ_location;
  run_manager_type<default_engine_type> run_manager;
};

template <class F>
int wrap(F &&f) {
  try {
    f();
    return 0;
  } catch (std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

}  // namespace

extern "C" {

const char *cem_plugin_last_error() { return g_err.c_str(); }

/// method: "canonical" or "semigrand_canonical". RT: (n_occ - 1) x n_occ.
void *cem_plugin_create(const char *method, cem_system *sys, int n_occ, const double *RT) {
  PluginCalc *p = nullptr;
  const int rc = wrap([&] {
    auto pc = std::make_unique<PluginCalc>();
    const std::string m(method ? method : "");
    if (m == "canonical") pc->calc.reset(make_GpuCanonicalCalculator());
    else if (m == "semigrand_canonical") pc->calc.reset(make_GpuSemiGrandCanonicalCalculator());
    else throw std::runtime_error("unknown method '" + m + "'");
    auto system = std::make_shared<system_type>();
    system->gpu_system = sys;
    system->n_occ = n_occ;
    system->param_RT.assign(RT, RT + (size_t)(n_occ - 1) * n_occ);
    pc->calc->reset(jsonParser{}, system);
    p = pc.release();
  });
  return rc == 0 ? p : nullptr;
}

void cem_plugin_destroy(void *h) { delete static_cast<PluginCalc *>(h); }

/// State: transformation matrix (row-major 3 x 3), occupation, conditions
/// (temperature; param_chem_pot of n_occ - 1 values for semi-grand runs).
int cem_plugin_set_state(void *h, const long *T, const int *occ, int64_t n_sites, double temperature,
                         const double *param_chem_pot) {
  return wrap([&] {
    auto *p = static_cast<PluginCalc *>(h);
    auto &st = p->state;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) st.configuration.transformation_matrix_to_super[a][b] = T[3 * a + b];
    st.configuration.occupation.assign(occ, occ + n_sites);
    st.conditions.scalar_values["temperature"] = temperature;
    const int nc = p->calc->system->n_occ - 1;
    if (param_chem_pot)
      st.conditions.vector_values["param_chem_pot"].assign(param_chem_pot, param_chem_pot + nc);
    p->occ_location.initialize(st.configuration.occupation, p->calc->system->n_occ);
    p->calc->set_state_and_potential(st, &p->occ_location);
  });
}

int cem_plugin_occ_delta(void *h, int n, const int64_t *sites, const int *new_occ, double *dE) {
  return wrap([&] {
    auto *p = static_cast<PluginCalc *>(h);
    std::vector<Index> s(sites, sites + n);
    std::vector<int> o(new_occ, new_occ + n);
    *dE = p->calc->potential->occ_delta_per_supercell(s, o);
  });
}

int cem_plugin_per_supercell(void *h, double *value) {
  return wrap([&] { *value = static_cast<PluginCalc *>(h)->calc->potential->per_supercell(); });
}

/// One run. seed < 0 leaves the run manager without an engine (the
/// reference's calculators reject that). requested precisions <= 0 are not
/// requested; none requested: a fixed run of max_count passes.
int cem_plugin_run(void *h, long long seed, long long max_count, long long n_equil,
                   long long check_period, double req_potential_energy, double req_param_composition,
                   int *occ_out, double *mean_potential, double *precision_potential,
                   long long *count, int *all_converged) {
  return wrap([&] {
    auto *p = static_cast<PluginCalc *>(h);
    auto &rm = p->run_manager;
    rm = run_manager_type<default_engine_type>{};
    if (seed >= 0) rm.engine = std::make_shared<default_engine_type>((unsigned long long)seed);
    rm.max_count = max_count;
    rm.n_equil = n_equil;
    rm.check_period = check_period;
    rm.min_count = 100;
    if (req_potential_energy > 0) rm.requested_abs_precision["potential_energy"] = req_potential_energy;
    if (req_param_composition > 0)
      rm.requested_abs_precision["param_composition"] = req_param_composition;
    p->calc->run(p->state, p->occ_location, rm);
    const auto &occ = p->state.configuration.occupation;
    std::copy(occ.begin(), occ.end(), occ_out);
    *mean_potential = rm.statistics.at("potential_energy")[0].mean;
    *precision_potential = rm.statistics.at("potential_energy")[0].calculated_precision;
    *count = rm.count;
    *all_converged = rm.all_converged ? 1 : 0;
  });
}

/// Species counts of the occupant lists (checks that run() kept them in
/// step with the state).
int cem_plugin_n_mol(void *h, int species, int64_t *n) {
  return wrap([&] { *n = static_cast<PluginCalc *>(h)->occ_location.n_mol(species); });
}

}  // extern "C"

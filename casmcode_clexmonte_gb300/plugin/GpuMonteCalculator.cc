// GPU Metropolis calculators behind the reference's calculator plugin
// interface: GpuCanonicalCalculator and GpuSemiGrandCanonicalCalculator
// derive from BaseMonteCalculator and are created by the factories
// make_GpuCanonicalCalculator / make_GpuSemiGrandCanonicalCalculator, the
// way the reference loads make_CanonicalCalculator
// (src/casm/clexmonte/monte_calculator/CanonicalCalculator.cc:580-586) and
// make_SemiGrandCanonicalCalculator (SemiGrandCanonicalCalculator.cc:517-523).
//
//   potential->occ_delta_per_supercell  -> cem_delta_energy
//     (CanonicalCalculator.cc:137-140; SemiGrandCanonicalCalculator.cc:186-213)
//   potential->per_supercell             -> cem_energy (minus n_uc mu . x)
//   run                                  -> cem_run in chunks of sampled
//     passes with the completion check of the run manager (the loop
//     occupation_metropolis_v2 runs, occupation_metropolis.hh:72-123, with
//     the default fixture's convergence criterion, CanonicalCalculator.cc:261-270)
//
// Every call goes through the C ABI of include/cem.h; the state keeps the
// reference's int occupations and is copied to and from the device's int8
// occupations at set_state_and_potential and at the end of run.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "cem.h"
#include "casm/clexmonte/monte_calculator/BaseMonteCalculator.hh"

namespace CASM {
namespace clexmonte {
namespace {

void ok(int rc, const char *what) {
  if (rc != CEM_OK && rc != CEM_STOPPED)
    throw std::runtime_error(std::string(what) + ": " + cem_last_error());
}

// Integrated autocorrelation time with Sokal's automatic window (smallest M
// with M >= 5 tau(M)), tau = 1/2 + sum_{t=1..M} rho(t).
double tau_int(const std::vector<double> &x, size_t begin) {
  const size_t n = x.size() - begin;
  if (n < 8) return 0.5;
  double m = 0.0;
  for (size_t i = begin; i < x.size(); ++i) m += x[i];
  m /= (double)n;
  double var = 0.0;
  for (size_t i = begin; i < x.size(); ++i) var += (x[i] - m) * (x[i] - m);
  var /= (double)n;
  if (var == 0.0) return 0.5;
  double tau = 0.5;
  for (size_t t = 1; t < n; ++t) {
    double c = 0.0;
    for (size_t i = begin; i + t < x.size(); ++i) c += (x[i] - m) * (x[i + t] - m);
    tau += c / ((double)n * var);
    if ((double)t >= 5.0 * tau) break;
  }
  return std::max(tau, 0.5);
}

// z(confidence) x standard error of the mean of x[begin:] corrected by 2 tau_int.
double calc_precision(const std::vector<double> &x, size_t begin, double z) {
  const size_t n = x.size() - begin;
  if (n < 2) return INFINITY;
  double m = 0.0;
  for (size_t i = begin; i < x.size(); ++i) m += x[i];
  m /= (double)n;
  double var = 0.0;
  for (size_t i = begin; i < x.size(); ++i) var += (x[i] - m) * (x[i] - m);
  var /= (double)n;
  return z * std::sqrt(2.0 * tau_int(x, begin) * var / (double)n);
}

// First sample after which x counts as equilibrated (-1 if none): the start
// of the first half moves forward one twentieth of the series at a time until
// the means of [start, N/2) and [N/2, N) agree within `precision` (the same
// two-partition test as the Python run fixture).
long long equilibration_index(const std::vector<double> &x, double precision) {
  const size_t n = x.size();
  if (n < 40) return -1;
  const size_t half = n / 2, step = std::max<size_t>(1, n / 20);
  double second = 0.0;
  for (size_t i = half; i < n; ++i) second += x[i];
  second /= (double)(n - half);
  for (size_t start = 0; start + step <= half; start += step) {
    double first = 0.0;
    for (size_t i = start; i < half; ++i) first += x[i];
    first /= (double)(half - start);
    if (std::fabs(first - second) <= precision) return (long long)start;
  }
  return -1;
}

// z with P(|Z| <= z) = confidence for a standard normal Z, by bisection on
// the normal CDF 0.5 erfc(-z / sqrt 2).
double z_of(double confidence) {
  const double p = 0.5 + 0.5 * confidence;
  double lo = 0.0, hi = 40.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (0.5 * std::erfc(-mid / std::sqrt(2.0)) < p) lo = mid;
    else hi = mid;
  }
  return 0.5 * (lo + hi);
}

}  // namespace

/// Potential of the state bound to the calculator's replica batch.
class GpuMontePotential : public BaseMontePotential {
 public:
  GpuMontePotential(std::shared_ptr<StateData> sd, cem_replicas *batch, bool semigrand,
                    std::shared_ptr<system_type> system)
      : BaseMontePotential(std::move(sd)), m_batch(batch), m_sgc(semigrand),
        m_system(std::move(system)) {}

  double per_supercell() override {
    double e = 0.0;
    std::vector<int64_t> counts(256);
    ok(cem_energy(m_batch, 0, &e, counts.data()), "per_supercell");
    if (!m_sgc) return e;
    // semi-grand potential: E_f - n_uc mu . x, x = R^T (N - N_origin) / n_uc
    const std::vector<int> &occ = state_data->state->configuration.occupation;
    const int no = m_system->n_occ;
    std::vector<double> dn(no, 0.0);
    for (int o : occ) dn[o] += 1.0;
    dn[0] -= (double)occ.size();
    const std::vector<double> &mu = state_data->state->conditions.vector_values.at("param_chem_pot");
    for (int k = 0; k < no - 1; ++k) {
      double x = 0.0;
      for (int a = 0; a < no; ++a) x += m_system->param_RT[k * no + a] * dn[a];
      e -= mu[k] * x;  // n_uc * mu * (x / n_uc)
    }
    return e;
  }

  double per_unitcell() override { return per_supercell() / (double)state_data->n_unitcells; }

  double occ_delta_per_supercell(std::vector<Index> const &linear_site_index,
                                 std::vector<int> const &new_occ) override {
    if (linear_site_index.size() != new_occ.size() || linear_site_index.empty())
      throw std::runtime_error("occ_delta_per_supercell: sites and new_occ differ in size");
    std::vector<int64_t> sites(linear_site_index.begin(), linear_site_index.end());
    std::vector<int32_t> occ(new_occ.begin(), new_occ.end());
    double de = 0.0;
    ok(cem_delta_energy(m_batch, 0, 1, (int)sites.size(), sites.data(), occ.data(), m_sgc ? 1 : 0,
                        &de, nullptr),
       "occ_delta_per_supercell");
    return de;
  }

 private:
  cem_replicas *m_batch;
  bool m_sgc;
  std::shared_ptr<system_type> m_system;
};

/// Shared implementation of the two methods.
class GpuMetropolisCalculator : public BaseMonteCalculator {
 public:
  GpuMetropolisCalculator(std::string name, bool semigrand)
      : BaseMonteCalculator(std::move(name)), m_sgc(semigrand) {}
  ~GpuMetropolisCalculator() override {
    if (m_batch) cem_replicas_destroy(m_batch);
  }

  Validator validate_state(state_type &state) const override {
    Validator v;
    const auto &c = state.conditions;
    if (!c.scalar_values.count("temperature")) v.error.insert("missing condition 'temperature'");
    if (m_sgc && !c.vector_values.count("param_chem_pot"))
      v.error.insert("missing condition 'param_chem_pot'");
    return v;
  }

  void set_state_and_potential(state_type &state, monte::OccLocation *occ_location) override {
    if (!system || !system->gpu_system)
      throw std::runtime_error("Error in " + calculator_name + ": no system (call reset first)");
    const Validator v = validate_state(state);
    if (!v.valid()) throw std::runtime_error("Error in " + calculator_name + ": " + *v.error.begin());
    // any supercell matrix: non-diagonal ones are indexed on their Hermite
    // normal form and support the potential (per_supercell,
    // occ_delta_per_supercell) and the semi-grand run(); the canonical run()
    // needs a diagonal supercell
    const auto &Tm = state.configuration.transformation_matrix_to_super;
    int64_t T[9], H[9];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) T[3 * a + b] = Tm[a][b];
    ok(cem_supercell_hnf(T, H), "set_state_and_potential");
    if (!m_batch || !std::equal(T, T + 9, m_T)) {
      if (m_batch) cem_replicas_destroy(m_batch);
      m_batch = nullptr;
      ok(cem_replicas_create_supercells(system->gpu_system, 1, T,
                                        m_sgc ? CEM_SEMIGRAND_CANONICAL : CEM_CANONICAL, &m_batch),
         "set_state_and_potential");
      std::copy(T, T + 9, m_T);
    }
    int64_t n_sites = 0;
    ok(cem_n_sites(m_batch, 0, &n_sites), "set_state_and_potential");
    const std::vector<int> &occ = state.configuration.occupation;
    if ((int64_t)occ.size() != n_sites)
      throw std::runtime_error("Error in " + calculator_name + ": occupation has " +
                               std::to_string(occ.size()) + " sites, the supercell " +
                               std::to_string(n_sites));
    std::vector<int8_t> o8(occ.size());
    for (size_t l = 0; l < occ.size(); ++l) {
      if (occ[l] < 0 || occ[l] >= system->n_occ)
        throw std::runtime_error("Error in " + calculator_name + ": occupant out of range");
      o8[l] = (int8_t)occ[l];
    }
    const double temperature = state.conditions.scalar_values.at("temperature");
    const double *mu = nullptr;
    if (m_sgc) mu = state.conditions.vector_values.at("param_chem_pot").data();
    ok(cem_set_conditions(m_batch, 0, temperature, mu), "set_state_and_potential");
    ok(cem_set_occupation(m_batch, 0, o8.data()), "set_state_and_potential");
    state_data = std::make_shared<StateData>();
    state_data->state = &state;
    state_data->occ_location = occ_location;
    state_data->n_unitcells = (Index)(H[0] * H[4] * H[8]);
    potential = std::make_shared<GpuMontePotential>(state_data, m_batch, m_sgc, system);
  }

  void run(state_type &state, monte::OccLocation &occ_location,
           run_manager_type<engine_type> &run_manager) override {
    this->set_state_and_potential(state, &occ_location);
    if (run_manager.engine == nullptr)
      throw std::runtime_error("Error in " + calculator_name + "::run: run_manager.engine==nullptr");
    this->engine = run_manager.engine;
    // the counter-based streams of the sweep are keyed by a seed drawn from
    // the run's engine
    ok(cem_set_seed(m_batch, 0, (*engine)()), "run");
    auto &rm = run_manager;
    if (rm.n_equil > 0) ok(cem_run(m_batch, rm.n_equil, rm.n_equil, 0), "run");
    ok(cem_reset_stats(m_batch), "run");
    const int nc = system->n_occ - 1;
    std::vector<double> e;
    std::vector<std::vector<double>> x(nc);
    const double z = z_of(rm.confidence);
    const bool check = !rm.requested_abs_precision.empty();
    long long count = rm.n_equil;
    rm.all_converged = false;
    long long eq_at = 0;
    std::map<std::string, std::vector<monte::BasicStatistics>> stats;
    const long long max_count = std::max(rm.max_count, rm.n_equil + 1);
    std::vector<double> pot, comp;
    while (count < max_count) {
      const long long chunk =
          check ? std::min(rm.check_period, max_count - count) : max_count - count;
      ok(cem_run(m_batch, chunk, 0, 1), "run");
      pot.assign(chunk, 0.0);
      comp.assign(chunk * nc, 0.0);
      int64_t got = 0;
      ok(cem_get_samples(m_batch, 0, pot.data(), comp.data(), chunk, &got), "run");
      for (int64_t s = 0; s < got; ++s) {
        e.push_back(pot[s]);
        for (int k = 0; k < nc; ++k) x[k].push_back(comp[s * nc + k]);
      }
      count += chunk;
      if (!check || (long long)e.size() < rm.min_count) continue;
      // completion check: every requested quantity equilibrated and within
      // its absolute precision over the equilibrated tail
      std::vector<std::pair<const std::vector<double> *, double>> series;
      auto it = rm.requested_abs_precision.find("potential_energy");
      if (it != rm.requested_abs_precision.end()) series.push_back({&e, it->second});
      it = rm.requested_abs_precision.find("param_composition");
      if (it != rm.requested_abs_precision.end())
        for (int k = 0; k < nc; ++k) series.push_back({&x[k], it->second});
      long long start = 0;
      bool equilibrated = true;
      for (auto &s : series) {
        const long long i = equilibration_index(*s.first, s.second);
        if (i < 0) equilibrated = false;
        start = std::max(start, i);
      }
      if (!equilibrated) continue;
      bool conv = true;
      for (auto &s : series) conv = conv && calc_precision(*s.first, (size_t)start, z) <= s.second;
      eq_at = start;
      if (conv) {
        rm.all_converged = true;
        break;
      }
    }
    // results over the equilibrated tail
    auto stat = [&](const std::vector<double> &v, const std::string &name) {
      monte::BasicStatistics b;
      double m = 0.0;
      for (size_t i = (size_t)eq_at; i < v.size(); ++i) m += v[i];
      b.mean = v.size() > (size_t)eq_at ? m / (double)(v.size() - eq_at) : NAN;
      b.calculated_precision = calc_precision(v, (size_t)eq_at, z);
      auto it = rm.requested_abs_precision.find(name);
      b.is_converged = it != rm.requested_abs_precision.end() && b.calculated_precision <= it->second;
      return b;
    };
    rm.statistics.clear();
    rm.statistics["potential_energy"] = {stat(e, "potential_energy")};
    for (int k = 0; k < nc; ++k) rm.statistics["param_composition"].push_back(stat(x[k], "param_composition"));
    rm.samples["potential_energy"] = {std::vector<double>(e.begin() + eq_at, e.end())};
    rm.count = count;
    rm.n_samples_for_equilibration = check ? eq_at : 0;
    // the evolved state back into the caller's configuration and lists
    std::vector<int8_t> o8(state.configuration.occupation.size());
    ok(cem_get_occupation(m_batch, 0, o8.data()), "run");
    for (size_t l = 0; l < o8.size(); ++l) state.configuration.occupation[l] = o8[l];
    occ_location.initialize(state.configuration.occupation, system->n_occ);
  }

 protected:
  bool m_sgc;
  cem_replicas *m_batch = nullptr;
  int64_t m_T[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};

 private:
  void _reset() override {
    if (m_batch) cem_replicas_destroy(m_batch);
    m_batch = nullptr;
  }
};

class GpuCanonicalCalculator : public GpuMetropolisCalculator {
 public:
  GpuCanonicalCalculator() : GpuMetropolisCalculator("GpuCanonicalCalculator", false) {}

 private:
  BaseMonteCalculator *_clone() const override {
    auto *c = new GpuCanonicalCalculator();
    c->params = params;
    c->system = system;
    return c;
  }
};

class GpuSemiGrandCanonicalCalculator : public GpuMetropolisCalculator {
 public:
  GpuSemiGrandCanonicalCalculator()
      : GpuMetropolisCalculator("GpuSemiGrandCanonicalCalculator", true) {}

 private:
  BaseMonteCalculator *_clone() const override {
    auto *c = new GpuSemiGrandCanonicalCalculator();
    c->params = params;
    c->system = system;
    return c;
  }
};

}  // namespace clexmonte
}  // namespace CASM

extern "C" {

CASM::clexmonte::BaseMonteCalculator *make_GpuCanonicalCalculator() {
  return new CASM::clexmonte::GpuCanonicalCalculator();
}

CASM::clexmonte::BaseMonteCalculator *make_GpuSemiGrandCanonicalCalculator() {
  return new CASM::clexmonte::GpuSemiGrandCanonicalCalculator();
}

}  // extern "C"

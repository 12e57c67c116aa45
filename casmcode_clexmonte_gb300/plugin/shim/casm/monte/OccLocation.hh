// Minimal stand-ins for the libcasm-monte types the Metropolis calculators
// touch (the package is not part of the reference sources): an occupation
// event, the per-species candidate lists (monte::OccLocation), the
// conditions value map, the state, and the run manager with its completion
// check parameters and results. Written for this project from the use the
// reference's calculators make of them (CanonicalCalculator.cc:413-462,
// occupation_metropolis.hh:72-123); only what the GPU adaptors need.
#pragma once

#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

namespace CASM {

typedef long Index;

namespace monte {

typedef std::mt19937_64 default_engine_type;

/// A series of occupation changes applied in order.
struct OccEvent {
  std::vector<Index> linear_site_index;
  std::vector<int> new_occ;
};

/// Sites holding each species: candidate lists a proposal draws from.
/// Removal swaps the last entry into the freed slot; insertion appends.
class OccLocation {
 public:
  void initialize(std::vector<int> const &occupation, int n_species) {
    m_loc.assign(n_species, {});
    m_pos.assign(occupation.size(), -1);
    for (Index l = 0; l < (Index)occupation.size(); ++l) {
      const int s = occupation[l];
      if (s < 0 || s >= n_species) throw std::runtime_error("OccLocation: occupant out of range");
      m_pos[l] = (Index)m_loc[s].size();
      m_loc[s].push_back(l);
    }
  }
  /// Apply `e` to `occupation` and the lists.
  void apply(OccEvent const &e, std::vector<int> &occupation) {
    for (size_t k = 0; k < e.linear_site_index.size(); ++k) {
      const Index l = e.linear_site_index[k];
      const int from = occupation[l], to = e.new_occ[k];
      if (from == to) continue;
      auto &src = m_loc[from];
      const Index last = src.back();
      src[m_pos[l]] = last;
      m_pos[last] = m_pos[l];
      src.pop_back();
      m_pos[l] = (Index)m_loc[to].size();
      m_loc[to].push_back(l);
      occupation[l] = to;
    }
  }
  Index n_mol(int species) const { return (Index)m_loc.at(species).size(); }
  Index mol_id(int species, Index i) const { return m_loc.at(species).at(i); }

 private:
  std::vector<std::vector<Index>> m_loc;
  std::vector<Index> m_pos;
};

/// Named scalar and vector values (conditions, properties).
struct ValueMap {
  std::map<std::string, double> scalar_values;
  std::map<std::string, std::vector<double>> vector_values;
};

template <typename ConfigType>
struct State {
  ConfigType configuration;
  ValueMap conditions;
};

/// Mean and calculated precision of one sampled quantity.
struct BasicStatistics {
  double mean = 0.0;
  double calculated_precision = 0.0;
  bool is_converged = false;
};

/// What a run needs from the run manager: the random engine, the completion
/// check (absolute precisions per quantity, checked every `check_period`
/// sampled passes once `min_count` passes have run, cut off at `max_count`),
/// and where it leaves its results.
template <typename EngineType>
struct RunManager {
  std::shared_ptr<EngineType> engine;
  long long n_equil = 0;
  long long max_count = 1000;
  long long min_count = 0;
  long long check_period = 100;
  double confidence = 0.95;
  std::map<std::string, double> requested_abs_precision;
  // results
  long long count = 0;
  long long n_samples_for_equilibration = -1;
  bool all_converged = false;
  std::map<std::string, std::vector<BasicStatistics>> statistics;
  std::map<std::string, std::vector<std::vector<double>>> samples;
};

}  // namespace monte
}  // namespace CASM

// The plugin interface of the reference's Monte Carlo calculators,
// restated for this project with the same class names and the signatures
// of the members the Metropolis methods use
// (include/casm/clexmonte/monte_calculator/BaseMonteCalculator.hh:26-264):
// BaseMontePotential (per_supercell, per_unitcell, occ_delta_per_supercell)
// and BaseMonteCalculator (reset, set_state_and_potential, run, clone).
// Value types the reference takes from libcasm-* (configuration, state, run
// manager, system, parameters) are the minimal stand-ins of OccLocation.hh
// and below; the sampling-function, analysis-function and event-data members
// are left out.
#pragma once

#include <array>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "../../monte/OccLocation.hh"

struct cem_system;

namespace CASM {
namespace clexmonte {

/// The configuration: supercell of the prim and one occupant index per site
/// (linear site index l = b * n_unitcells + unitcell).
struct Configuration {
  std::array<std::array<long, 3>, 3> transformation_matrix_to_super{};
  std::vector<int> occupation;
};

typedef Configuration config_type;
typedef monte::State<config_type> state_type;
typedef monte::default_engine_type default_engine_type;
template <typename EngineType>
using run_manager_type = monte::RunManager<EngineType>;

/// System data: the cluster expansion on the device (cem_system_create), the
/// occupants per site and R^T = dparam_dmol ((n_occ - 1) x n_occ).
struct System {
  cem_system *gpu_system = nullptr;
  int n_sublat = 1;
  int n_occ = 2;
  std::vector<double> param_RT;
};
typedef System system_type;

/// Calculator method parameters (flat key -> number).
typedef std::map<std::string, double> jsonParser;

struct Validator {
  std::set<std::string> error, warning;
  bool valid() const { return error.empty(); }
};

/// State data the potential reads: the state, its occupant locations and its
/// number of unit cells.
struct StateData {
  state_type *state = nullptr;
  monte::OccLocation *occ_location = nullptr;
  Index n_unitcells = 0;
};

/// Potential of the current state (formation energy for canonical runs, the
/// semi-grand potential for semi-grand canonical runs).
class BaseMontePotential {
 public:
  explicit BaseMontePotential(std::shared_ptr<StateData> _state_data)
      : state_data(std::move(_state_data)) {}
  virtual ~BaseMontePotential() = default;

  std::shared_ptr<StateData> state_data;

  /// Value for the whole supercell.
  virtual double per_supercell() = 0;

  /// Value per unit cell.
  virtual double per_unitcell() = 0;

  /// Supercell value change when the listed sites take the listed occupants,
  /// one after the other.
  virtual double occ_delta_per_supercell(std::vector<Index> const &linear_site_index,
                                         std::vector<int> const &new_occ) = 0;
};

/// A Monte Carlo method, loaded from a plugin library by its make_<Name>
/// factory.
class BaseMonteCalculator {
 public:
  typedef default_engine_type engine_type;

  explicit BaseMonteCalculator(std::string _calculator_name)
      : engine(std::make_shared<engine_type>()), calculator_name(std::move(_calculator_name)) {}
  virtual ~BaseMonteCalculator() = default;

  std::shared_ptr<engine_type> engine;  // never null
  std::string calculator_name;
  jsonParser params;                     // method parameters
  std::shared_ptr<system_type> system;

  /// Store parameters and system, then let the method reset itself.
  void reset(jsonParser const &_params, std::shared_ptr<system_type> _system) {
    this->params = _params;
    this->system = std::move(_system);
    this->_reset();
  }

  /// Errors and warnings about a state's conditions and configuration.
  virtual Validator validate_state(state_type &state) const = 0;

  std::shared_ptr<StateData> state_data;         // of the current state
  std::shared_ptr<BaseMontePotential> potential;  // of the current state

  /// Check and adopt `state`; builds state_data and potential.
  virtual void set_state_and_potential(state_type &state, monte::OccLocation *occ_location) = 0;

  /// One run at the state's conditions; the state and the occupant lists
  /// are updated in place, the results go to the run manager.
  virtual void run(state_type &state, monte::OccLocation &occ_location,
                   run_manager_type<engine_type> &run_manager) = 0;

  std::unique_ptr<BaseMonteCalculator> clone() const {
    return std::unique_ptr<BaseMonteCalculator>(this->_clone());
  }

 private:
  virtual void _reset() = 0;
  virtual BaseMonteCalculator *_clone() const = 0;
};

}  // namespace clexmonte
}  // namespace CASM

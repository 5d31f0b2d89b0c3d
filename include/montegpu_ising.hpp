// montegpu_ising.hpp -- header-only C++ form of libcasm-monte's 2-D Ising model and its
// semi-grand canonical pieces, with the Metropolis passes run on the GPU through the C-ABI.
//
// Same names, argument meaning and arithmetic as the reference's C++:
//   include/casm/monte/ising_cpp/model.hh:19-452        IsingConfiguration, IsingState,
//                                                      IsingFormationEnergy,
//                                                      IsingParamComposition, IsingSystem
//   include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:36-321
//                                                      SemiGrandCanonicalConditions,
//                                                      SemiGrandCanonicalPotential,
//                                                      SemiGrandCanonicalEventGenerator
//   include/casm/monte/RandomNumberGenerator.hh:15-42  RandomNumberGenerator
// Eigen vectors become std::vector (occupation: int, +1/-1, column-major l = shape[0]*j + i).
// Energies are accumulated in the reference's order, so host values are bit-identical.
// The reference's constructors ignore a state passed to them (they test the member, not the
// argument); here a non-null state is set, as their documentation says.
//
// run_metropolis_passes() replaces the host loop of basic_occupation_metropolis for this
// model: the GPU consumes the engine's own draws (random_int(N-1), then random_real(1.0) for
// uphill steps) and hands the advanced engine back, so the trajectory equals the host loop's.
//
// SemiGrandCanonicalCalculator<System, EventGenerator>::run (basic_semigrand_canonical.hh:
// 322-470) with the sampling-function factories of :476-627: for IsingSystem with the
// built-in SemiGrandCanonicalEventGenerator the passes run on the GPU as a serial replay,
// with the completion check evaluated exactly as the reference evaluates it before every step
// (samples and counts change only at pass boundaries, so a launch ends at the first pass
// boundary where that check could end the run or run a convergence check); any other system
// or event generator runs the reference's generic loop (montegpu_methods.hpp) on the host.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <type_traits>

#include "montegpu.h"
#include "montegpu_methods.hpp"

namespace montegpu {
namespace ising_cpp {

typedef long Index;

/// Boltzmann constant (eV/K), the value of the reference's definitions.
constexpr double KB = 8.6173303e-05;

struct ValueMap {
  std::map<std::string, bool> boolean_values;
  std::map<std::string, double> scalar_values;
  std::map<std::string, std::vector<double>> vector_values;
};

using monte::RandomNumberGenerator;

struct OccEvent {
  std::vector<Index> linear_site_index;
  std::vector<int> new_occ;
};

class IsingConfiguration {
 public:
  IsingConfiguration() : IsingConfiguration(std::vector<int>{0, 0}, 1) {}
  /// JSON text {"shape": [...], "occupation": [...]} (model.hh:133-138)
  std::string to_json() const {
    std::ostringstream ss;
    ss << "{\"shape\": [" << shape[0] << ", " << shape[1] << "], \"occupation\": [";
    for (size_t k = 0; k < m_occupation.size(); ++k) ss << (k ? ", " : "") << m_occupation[k];
    ss << "]}";
    return ss.str();
  }
  explicit IsingConfiguration(std::vector<int> _shape, int fill_value = 1) : shape(_shape) {
    if (shape.size() != 2) throw std::runtime_error("IsingConfiguration only supports 2d");
    m_occupation.assign(static_cast<size_t>(shape[0]) * shape[1], fill_value);
    n_sites = n_variable_sites = n_unitcells = static_cast<Index>(m_occupation.size());
  }
  std::vector<int> shape;
  Index n_sites = 0;
  Index n_variable_sites = 0;
  Index n_unitcells = 0;

  std::vector<int> const& occupation() const { return m_occupation; }
  void set_occupation(std::vector<int> const& occupation) {
    if (occupation.size() != m_occupation.size())
      throw std::runtime_error("Error in IsingConfiguration::set_occupation: size mismatch");
    m_occupation = occupation;
  }
  int occ(Index linear_site_index) const { return m_occupation[linear_site_index]; }
  void set_occ(Index linear_site_index, int new_occ) { m_occupation[linear_site_index] = new_occ; }
  Index within(Index index, int dim) const {
    Index r = index % shape[dim];
    return r < 0 ? r + shape[dim] : r;
  }
  std::vector<int> from_linear_site_index(Index l) const {
    return {static_cast<int>(l % shape[0]), static_cast<int>(l / shape[0])};
  }
  Index to_linear_site_index(Index row, Index col) const { return shape[0] * col + row; }

 private:
  std::vector<int> m_occupation;
};

class IsingState {
 public:
  IsingState(IsingConfiguration _configuration, ValueMap _conditions, ValueMap _properties = ValueMap())
      : configuration(std::move(_configuration)), conditions(std::move(_conditions)),
        properties(std::move(_properties)) {}
  IsingConfiguration configuration;
  ValueMap conditions;
  ValueMap properties;
};

class IsingFormationEnergy {
 public:
  typedef IsingState state_type;
  IsingFormationEnergy(double _J = 1.0, int _lattice_type = 1, bool _use_nlist = true,
                       state_type const* _state = nullptr)
      : J(_J), lattice_type(_lattice_type), state(nullptr), m_use_nlist(_use_nlist) {
    if (lattice_type != 1) throw std::runtime_error("Unsupported lattice_type");
    if (_state != nullptr) set_state(_state);
  }
  double J;
  int lattice_type;
  state_type const* state;

  /// Forward neighbours (+i, +j) for the energy, all four for a flip.
  void set_state(state_type const* _state) {
    if (_state == nullptr) throw std::runtime_error("Error in IsingFormationEnergy::set_state: _state==nullptr");
    state = _state;
    if (!m_use_nlist) return;
    IsingConfiguration const& c = state->configuration;
    m_nlist.assign(c.n_sites, {});
    m_flower.assign(c.n_sites, {});
    for (Index l = 0; l < c.n_sites; ++l) {
      const std::vector<int> ij = c.from_linear_site_index(l);
      const Index i = ij[0], j = ij[1];
      const Index ip = c.to_linear_site_index(c.within(i + 1, 0), j);
      const Index jp = c.to_linear_site_index(i, c.within(j + 1, 1));
      m_nlist[l] = {ip, jp};
      m_flower[l] = {ip, jp, c.to_linear_site_index(c.within(i - 1, 0), j),
                     c.to_linear_site_index(i, c.within(j - 1, 1))};
    }
  }

  double per_supercell() const {
    IsingConfiguration const& c = state->configuration;
    std::vector<int> const& s = c.occupation();
    double e = 0.0;
    if (m_use_nlist) {
      for (Index l = 0; l < c.n_sites; ++l) e += s[l] * (s[m_nlist[l][0]] + s[m_nlist[l][1]]);
      e *= -J;
      return e;
    }
    const Index rows = c.shape[0], cols = c.shape[1];
    for (Index i = 0; i < rows; ++i) {  // row i . row i+1
      const Index ip = c.within(i + 1, 0);
      long dot = 0;
      for (Index j = 0; j < cols; ++j) dot += s[c.to_linear_site_index(i, j)] * s[c.to_linear_site_index(ip, j)];
      e += -J * dot;
    }
    for (Index j = 0; j < cols; ++j) {  // column j . column j+1
      const Index jp = c.within(j + 1, 1);
      long dot = 0;
      for (Index i = 0; i < rows; ++i) dot += s[c.to_linear_site_index(i, j)] * s[c.to_linear_site_index(i, jp)];
      e += -J * dot;
    }
    return e;
  }
  double per_unitcell() const { return per_supercell() / state->configuration.n_unitcells; }

  double occ_delta_per_supercell(std::vector<Index> const& linear_site_index, std::vector<int> const& new_occ) const {
    if (linear_site_index.size() == 1) return single_delta(linear_site_index[0], new_occ[0]);
    // several sites: each change applied in turn, then undone
    auto& c = const_cast<IsingConfiguration&>(state->configuration);
    double dE = 0.0;
    std::vector<int> original;
    for (size_t k = 0; k < linear_site_index.size(); ++k) {
      dE += single_delta(linear_site_index[k], new_occ[k]);
      original.push_back(c.occ(linear_site_index[k]));
      c.set_occ(linear_site_index[k], new_occ[k]);
    }
    for (size_t k = 0; k < original.size(); ++k) c.set_occ(linear_site_index[k], original[k]);
    return dE;
  }

 private:
  double single_delta(Index l, int new_occ) const {
    IsingConfiguration const& c = state->configuration;
    std::vector<int> const& s = c.occupation();
    if (m_use_nlist) {
      auto const& n = m_flower[l];
      return -J * (new_occ - s[l]) * (s[n[0]] + s[n[1]] + s[n[2]] + s[n[3]]);
    }
    const std::vector<int> ij = c.from_linear_site_index(l);
    const Index i = ij[0], j = ij[1];
    const double ds = new_occ - s[l];
    return -J * ds *
           (s[c.to_linear_site_index(i, c.within(j - 1, 1))] + s[c.to_linear_site_index(i, c.within(j + 1, 1))] +
            s[c.to_linear_site_index(c.within(i - 1, 0), j)] + s[c.to_linear_site_index(c.within(i + 1, 0), j)]);
  }
  bool m_use_nlist = true;

 public:
  bool uses_nlist() const { return m_use_nlist; }

 private:
  std::vector<std::vector<Index>> m_nlist;
  std::vector<std::vector<Index>> m_flower;
};

class IsingParamComposition {
 public:
  typedef IsingState state_type;
  explicit IsingParamComposition(state_type const* _state = nullptr) : state(nullptr) {
    if (_state != nullptr) set_state(_state);
  }
  state_type const* state;
  void set_state(state_type const* _state) {
    if (_state == nullptr) throw std::runtime_error("Error in IsingParamComposition::set_state: _state==nullptr");
    state = _state;
  }
  Index n_independent_compositions() const { return 1; }
  /// N x = (N + sum s) / 2
  std::vector<double> per_supercell() const {
    std::vector<int> const& s = state->configuration.occupation();
    long sum = 0;
    for (int v : s) sum += v;
    return {static_cast<double>(static_cast<long>(s.size()) + sum) / 2.0};
  }
  std::vector<double> per_unitcell() const {
    return {per_supercell()[0] / state->configuration.n_unitcells};
  }
  std::vector<double> occ_delta_per_supercell(std::vector<Index> const& linear_site_index,
                                              std::vector<int> const& new_occ) const {
    double Ndx = 0.0;
    for (size_t k = 0; k < linear_site_index.size(); ++k)
      Ndx += (new_occ[k] - state->configuration.occ(linear_site_index[k])) / 2.0;
    return {Ndx};
  }
};

class IsingSystem {
 public:
  typedef IsingState state_type;
  typedef IsingFormationEnergy formation_energy_f_type;
  typedef IsingParamComposition param_composition_f_type;
  IsingSystem(formation_energy_f_type _formation_energy_calculator,
              param_composition_f_type _param_composition_calculator)
      : formation_energy_calculator(std::move(_formation_energy_calculator)),
        param_composition_calculator(std::move(_param_composition_calculator)) {}
  formation_energy_f_type formation_energy_calculator;
  param_composition_f_type param_composition_calculator;
};

namespace semigrand_canonical {

class SemiGrandCanonicalConditions {
 public:
  SemiGrandCanonicalConditions(double _temperature, std::vector<double> _exchange_potential)
      : temperature(_temperature), exchange_potential(std::move(_exchange_potential)) {
    if (temperature <= 0.0) throw std::runtime_error("Error in SemiGrandCanonicalConditions: temperature <= 0");
    beta = 1.0 / (KB * temperature);
  }
  /// From "temperature" (scalar) and "exchange_potential" (vector).
  static SemiGrandCanonicalConditions from_values(ValueMap const& values) {
    auto t = values.scalar_values.find("temperature");
    if (t == values.scalar_values.end())
      throw std::runtime_error("Error in SemiGrandCanonicalConditions: missing \"temperature\"");
    auto mu = values.vector_values.find("exchange_potential");
    if (mu == values.vector_values.end())
      throw std::runtime_error("Error in SemiGrandCanonicalConditions: missing \"exchange_potential\"");
    return SemiGrandCanonicalConditions(t->second, mu->second);
  }
  double temperature;
  std::vector<double> exchange_potential;
  double beta;
};

/// E_sgc = E_f - mu . N x, and its change for an event.
class SemiGrandCanonicalPotential {
 public:
  typedef IsingState state_type;
  explicit SemiGrandCanonicalPotential(std::shared_ptr<IsingSystem> _system) : system(_system) {
    if (!system) throw std::runtime_error("Error constructing SemiGrandCanonicalPotential: _system==nullptr");
  }
  void set_state(state_type const* _state, std::shared_ptr<SemiGrandCanonicalConditions> _conditions) {
    if (_state == nullptr) throw std::runtime_error("Error in SemiGrandCanonicalPotential::set_state: _state==nullptr");
    state = _state;
    conditions = _conditions;
    system->formation_energy_calculator.set_state(state);
    system->param_composition_calculator.set_state(state);
  }
  double per_supercell() const {
    const std::vector<double> Nx = system->param_composition_calculator.per_supercell();
    return system->formation_energy_calculator.per_supercell() - dot(conditions->exchange_potential, Nx);
  }
  double per_unitcell() const { return per_supercell() / state->configuration.n_unitcells; }
  double occ_delta_per_supercell(std::vector<Index> const& linear_site_index, std::vector<int> const& new_occ) const {
    const double dEf = system->formation_energy_calculator.occ_delta_per_supercell(linear_site_index, new_occ);
    const std::vector<double> Ndx = system->param_composition_calculator.occ_delta_per_supercell(linear_site_index, new_occ);
    return dEf - dot(conditions->exchange_potential, Ndx);
  }
  double occ_delta_per_supercell(OccEvent const& e) const {
    return occ_delta_per_supercell(e.linear_site_index, e.new_occ);
  }
  std::shared_ptr<IsingSystem> system;
  state_type const* state = nullptr;
  std::shared_ptr<SemiGrandCanonicalConditions> conditions;

 private:
  static double dot(std::vector<double> const& a, std::vector<double> const& b) {
    double r = 0.0;
    for (size_t k = 0; k < a.size() && k < b.size(); ++k) r = (k == 0) ? a[k] * b[k] : r + a[k] * b[k];
    return r;
  }
};

/// One random site, flipped: l = random_int(N - 1), new_occ = -occ(l).
template <typename EngineType = std::mt19937_64>
class SemiGrandCanonicalEventGenerator {
 public:
  typedef IsingState state_type;
  typedef EngineType engine_type;
  typedef RandomNumberGenerator<EngineType> random_number_generator_type;
  void set_state(state_type* _state) {
    if (_state == nullptr) throw std::runtime_error("Error in SemiGrandCanonicalEventGenerator::set_state: _state==nullptr");
    state = _state;
    occ_event.linear_site_index.assign(1, 0);
    occ_event.new_occ.assign(1, 0);
  }
  OccEvent const& propose(RandomNumberGenerator<EngineType>& random_number_generator) {
    const Index l = random_number_generator.random_int(state->configuration.n_variable_sites - 1);
    occ_event.linear_site_index[0] = l;
    occ_event.new_occ[0] = -state->configuration.occ(l);
    return occ_event;
  }
  void apply(OccEvent const& e) {
    for (size_t k = 0; k < e.linear_site_index.size(); ++k) state->configuration.set_occ(e.linear_site_index[k], e.new_occ[k]);
  }
  state_type* state = nullptr;
  OccEvent occ_event;
};

struct MetropolisCounts {
  unsigned long long n_accept = 0;
  unsigned long long n_reject = 0;
};

/// n_passes Metropolis passes of n_variable_sites steps each on the GPU, for the state under
/// the potential's conditions, drawing from (and advancing) `engine` exactly as the host loop
/// of basic_occupation_metropolis would; the state's occupation is updated in place.
inline MetropolisCounts run_metropolis_passes(IsingState& state, SemiGrandCanonicalPotential const& potential,
                                              int n_passes, std::mt19937_64& engine, bool use_nlist = true) {
  IsingConfiguration& c = state.configuration;
  const double J = potential.system->formation_energy_calculator.J;
  const double T = potential.conditions->temperature;
  const double mu = potential.conditions->exchange_potential.at(0);
  std::ostringstream es;
  es << engine;
  const std::string est = es.str();
  const char* states[1] = {est.c_str()};
  std::vector<int32_t> occ(c.occupation().begin(), c.occupation().end());
  mg_ising_replay* h = nullptr;
  if (mg_ising_replay_create(c.shape[0], c.shape[1], 1, use_nlist ? 1 : 0, &J, &T, &mu, occ.data(), states, &h) != 0)
    throw std::runtime_error(mg_last_error());
  MetropolisCounts counts;
  std::vector<long long> samples(2 + c.shape[0] + c.shape[1]);
  int n_samples = 0;
  int status = mg_ising_replay_run(h, n_passes, n_passes > 0 ? n_passes : 1, samples.data(), 1, &n_samples);
  std::vector<char> buf(est.size() + 4096);
  char* out_states[1] = {buf.data()};
  if (status == 0) status = mg_ising_replay_get_state(h, occ.data(), out_states, buf.size(), &counts.n_accept,
                                                      &counts.n_reject);
  std::string err = status != 0 ? std::string(mg_last_error()) : std::string();
  mg_ising_replay_destroy(h);
  if (status != 0) throw std::runtime_error(err);
  c.set_occupation(std::vector<int>(occ.begin(), occ.end()));
  std::istringstream is(std::string(buf.data()));
  is >> engine;
  return counts;
}

typedef monte::methods::BasicOccupationMetropolisData<monte::BasicStatistics> SemiGrandCanonicalData;

/// Semi-grand canonical Metropolis calculator (basic_semigrand_canonical.hh:322-470).
template <typename SystemType = IsingSystem,
          typename EventGeneratorType = SemiGrandCanonicalEventGenerator<std::mt19937_64>>
class SemiGrandCanonicalCalculator {
 public:
  typedef SystemType system_type;
  typedef typename system_type::state_type state_type;
  typedef typename system_type::formation_energy_f_type formation_energy_f_type;
  typedef typename system_type::param_composition_f_type param_composition_f_type;
  typedef SemiGrandCanonicalPotential potential_type;
  typedef EventGeneratorType event_generator_type;
  typedef typename event_generator_type::engine_type engine_type;
  typedef typename event_generator_type::random_number_generator_type random_number_generator_type;

  explicit SemiGrandCanonicalCalculator(std::shared_ptr<system_type> _system)
      : system(_system ? _system
                       : throw std::runtime_error("Error constructing SemiGrandCanonicalCalculator: _system==nullptr")),
        state(nullptr), conditions(nullptr), potential(_system),
        formation_energy_calculator(&potential.system->formation_energy_calculator),
        param_composition_calculator(&potential.system->param_composition_calculator) {}

  std::shared_ptr<system_type> system;
  state_type* state;
  std::shared_ptr<SemiGrandCanonicalConditions> conditions;
  potential_type potential;
  formation_energy_f_type* formation_energy_calculator;
  param_composition_f_type* param_composition_calculator;
  std::shared_ptr<SemiGrandCanonicalData> data;
  /// device time of the GPU passes of the last run (ms; 0 for a host run)
  double last_kernel_ms = 0.0;
  /// most passes per GPU launch
  int max_passes_per_launch = 4096;

  /// Run at the state's conditions until the completion check ends it; `state` is modified in
  /// place and the engine advanced.  write_status_f(calculator, method_log) is called when a
  /// status is due and at the end.
  template <typename WriteStatusF>
  std::shared_ptr<SemiGrandCanonicalData> run(state_type& state,
                                              monte::StateSamplingFunctionMap const& sampling_functions,
                                              monte::jsonStateSamplingFunctionMap const& json_sampling_functions,
                                              monte::CompletionCheckParams<monte::BasicStatistics> const& completion_check_params,
                                              event_generator_type event_generator, int sample_period,
                                              std::optional<monte::MethodLog> method_log,
                                              std::shared_ptr<engine_type> random_engine, WriteStatusF write_status_f) {
    this->state = &state;
    this->conditions = std::make_shared<SemiGrandCanonicalConditions>(
        SemiGrandCanonicalConditions::from_values(this->state->conditions));
    const double temperature = this->conditions->temperature;
    const monte::CountType n_steps_per_pass = this->state->configuration.n_variable_sites;
    this->potential.set_state(this->state, this->conditions);
    event_generator.set_state(this->state);
    this->data = std::make_shared<SemiGrandCanonicalData>(sampling_functions, json_sampling_functions,
                                                          n_steps_per_pass, completion_check_params);
    last_kernel_ms = 0.0;
    if (!random_engine) {
      random_engine = std::make_shared<engine_type>();
      std::random_device device;
      random_engine->seed(device());
    }
    if (!method_log.has_value()) {
      method_log = monte::MethodLog();
      method_log->logfile_path = "status.json";
      method_log->log_frequency = 600.0;
    }
    if constexpr (std::is_same<system_type, IsingSystem>::value &&
                  std::is_same<event_generator_type, SemiGrandCanonicalEventGenerator<std::mt19937_64>>::value) {
      method_log->log.restart_clock();
      method_log->log.begin_lap();
      gpu_replay(sample_period, *method_log, *random_engine, write_status_f);
      write_status_f(*this, *method_log);
    } else {
      auto dpotential_f = [this](OccEvent const& e) { return this->potential.occ_delta_per_supercell(e); };
      auto propose_event_f = [&](random_number_generator_type& rng) -> OccEvent const& {
        return event_generator.propose(rng);
      };
      auto apply_event_f = [&](OccEvent const& e) -> void { event_generator.apply(e); };
      auto _write_status_f = [&](SemiGrandCanonicalData const&, monte::MethodLog& log) { write_status_f(*this, log); };
      monte::methods::basic_occupation_metropolis(*this->data, temperature, dpotential_f, propose_event_f,
                                                  apply_event_f, sample_period, method_log, random_engine,
                                                  _write_status_f);
    }
    return this->data;
  }

  /// run() writing no status
  std::shared_ptr<SemiGrandCanonicalData> run(state_type& state,
                                              monte::StateSamplingFunctionMap const& sampling_functions,
                                              monte::jsonStateSamplingFunctionMap const& json_sampling_functions,
                                              monte::CompletionCheckParams<monte::BasicStatistics> const& completion_check_params,
                                              event_generator_type event_generator, int sample_period = 1,
                                              std::optional<monte::MethodLog> method_log = std::nullopt,
                                              std::shared_ptr<engine_type> random_engine = nullptr) {
    return run(state, sampling_functions, json_sampling_functions, completion_check_params, event_generator,
               sample_period, method_log, random_engine,
               [](SemiGrandCanonicalCalculator const&, monte::MethodLog& log) { log.log.begin_lap(); });
  }

 private:
  // The main loop of basic_occupation_metropolis.hh:381-422 for the built-in model, as a GPU
  // serial replay in chunks of whole passes; the completion check is called once per pass
  // boundary and its N - 1 further calls of the pass are applied with repeat_calls.
  template <typename WriteStatusF>
  void gpu_replay(int sample_period, monte::MethodLog& method_log, engine_type& engine, WriteStatusF& write_status_f) {
    SemiGrandCanonicalData& d = *this->data;
    IsingConfiguration& cfg = this->state->configuration;
    const int rows = cfg.shape[0], cols = cfg.shape[1];
    const monte::CountType N = cfg.n_variable_sites;
    const double J = this->system->formation_energy_calculator.J;
    const bool use_nlist = this->system->formation_energy_calculator.uses_nlist();
    if (this->conditions->exchange_potential.size() != 1)
      throw std::runtime_error("Error in SemiGrandCanonicalCalculator::run: exchange_potential must have size 1");
    const double mu = this->conditions->exchange_potential[0];
    const double T = this->conditions->temperature;
    if (sample_period < 1) throw std::runtime_error("Error in SemiGrandCanonicalCalculator::run: sample_period < 1");
    std::ostringstream es;
    es << engine;
    const std::string est = es.str();
    const char* states[1] = {est.c_str()};
    std::vector<int32_t> occ(cfg.occupation().begin(), cfg.occupation().end());
    mg_ising_replay* h = nullptr;
    if (mg_ising_replay_create(rows, cols, 1, use_nlist ? 1 : 0, &J, &T, &mu, occ.data(), states, &h) != MG_OK)
      throw std::runtime_error(mg_last_error());
    std::string err;
    try {
      main_loop(h, d, N, rows, cols, J, mu, use_nlist, sample_period, method_log, write_status_f);
    } catch (std::exception const& e) {
      err = e.what();
    }
    // bring the occupation, the engine and the counts back (also after an error)
    std::vector<char> buf(est.size() + 8192);
    char* out_states[1] = {buf.data()};
    unsigned long long acc = 0, rej = 0;
    const int st = mg_ising_replay_get_state(h, occ.data(), out_states, buf.size(), &acc, &rej);
    if (st != MG_OK && err.empty()) err = mg_last_error();
    mg_ising_replay_destroy(h);
    if (!err.empty()) throw std::runtime_error(err);
    cfg.set_occupation(std::vector<int>(occ.begin(), occ.end()));
    std::istringstream is(std::string(buf.data()));
    is >> engine;
    d.n_accept = acc;
    d.n_reject = rej;
  }

  template <typename WriteStatusF>
  void main_loop(mg_ising_replay* h, SemiGrandCanonicalData& d, monte::CountType N, int rows, int cols, double J,
                 double mu, bool use_nlist, int sample_period, monte::MethodLog& method_log,
                 WriteStatusF& write_status_f) {
    auto& cc = d.completion_check;
    bool device_only = d.json_sampling_functions.empty();
    for (auto const& pair : d.sampling_functions)
      device_only &= pair.second.device_owner == this && !pair.second.device_quantity.empty();
    int max_chunk = std::max(1, max_passes_per_launch);
    if (cc.params().cutoff_params.max_clocktime.has_value()) max_chunk = std::min(max_chunk, sample_period);
    const int stride = 2 + rows + cols;
    monte::CountType n_samples_now = 0;
    auto check = [&]() { return cc.is_complete(d.samplers, d.sample_weight, d.n_pass, method_log.log); };
    bool complete = check();
    while (!complete) {
      cc.repeat_calls(N - 1);
      // the chunk: up to the first pass boundary at which the check could act
      int k = 0;
      monte::CountType ns = n_samples_now;
      int limit = device_only ? max_chunk
                              : (int)std::max<monte::CountType>(1, sample_period - (d.n_pass % sample_period));
      limit = std::min(limit, max_chunk);
      while (k < limit) {
        ++k;
        const monte::CountType p = d.n_pass + k;
        if (p % sample_period == 0) ++ns;
        if (cc.could_complete_at(ns, p)) break;
      }
      const monte::CountType expected = (d.n_pass + k) / sample_period - d.n_pass / sample_period;
      std::vector<long long> buf((size_t)std::max<monte::CountType>(expected, 1) * stride);
      int n_written = 0;
      if (mg_ising_replay_run(h, k, sample_period, buf.data(), (int)std::max<monte::CountType>(expected, 1),
                              &n_written) != MG_OK)
        throw std::runtime_error(mg_last_error());
      float ms = 0.f;
      mg_ising_replay_last_kernel_ms(h, &ms);
      last_kernel_ms += ms;
      int si = 0;
      for (int b = 0; b < k; ++b) {
        d.n_pass += 1;
        if (d.n_pass % sample_period == 0) {
          push_sample(h, d, &buf[(size_t)si * stride], N, rows, cols, J, mu, use_nlist, device_only);
          ++si;
          ++n_samples_now;
          if (method_log.log_frequency.has_value() && method_log.log.lap_time() >= method_log.log_frequency.value())
            write_status_f(*this, method_log);
        }
        complete = check();
        if (complete) {
          if (b != k - 1) throw std::runtime_error("internal error: completion inside a planned chunk");
          break;
        }
        if (b < k - 1) cc.repeat_calls(N - 1);
      }
    }
  }

  // One sample from the device's integer sums (spin sum, bond sum or row/column dot products)
  // in the reference's arithmetic order; other sampling functions read the host state, which
  // is brought back from the device first.
  void push_sample(mg_ising_replay* h, SemiGrandCanonicalData& d, const long long* row, monte::CountType N, int rows,
                   int cols, double J, double mu, bool use_nlist, bool device_only) {
    const long long spin_sum = row[0], bond_sum = row[1];
    const double Nx = static_cast<double>(N + spin_sum) / 2.0;
    double ef;
    if (use_nlist) {
      ef = static_cast<double>(bond_sum);
      ef *= -J;
    } else {
      ef = 0.0;
      for (int i = 0; i < rows; ++i) ef += -J * static_cast<double>(row[2 + i]);
      for (int j = 0; j < cols; ++j) ef += -J * static_cast<double>(row[2 + rows + j]);
    }
    if (!device_only) {
      std::vector<int32_t> occ((size_t)N);
      if (mg_ising_replay_get_state(h, occ.data(), nullptr, 0, nullptr, nullptr) != MG_OK)
        throw std::runtime_error(mg_last_error());
      this->state->configuration.set_occupation(std::vector<int>(occ.begin(), occ.end()));
    }
    for (auto const& pair : d.sampling_functions) {
      auto const& f = pair.second;
      if (f.device_owner == this && f.device_quantity == "param_composition") {
        d.samplers.at(f.name)->push_back(std::vector<double>{Nx / static_cast<double>(N)});
      } else if (f.device_owner == this && f.device_quantity == "formation_energy") {
        d.samplers.at(f.name)->push_back(std::vector<double>{ef / static_cast<double>(N)});
      } else if (f.device_owner == this && f.device_quantity == "potential_energy") {
        d.samplers.at(f.name)->push_back(std::vector<double>{(ef - mu * Nx) / static_cast<double>(N)});
      } else {
        d.samplers.at(f.name)->push_back(f());
      }
    }
    for (auto const& pair : d.json_sampling_functions)
      d.json_samplers.at(pair.second.name).values.push_back(pair.second());
  }
};

/// Parametric composition per unit cell (basic_semigrand_canonical.hh:486-517).
template <typename CalculatorType>
monte::StateSamplingFunction make_parametric_composition_f(std::shared_ptr<CalculatorType> mc_calculator) {
  if (mc_calculator == nullptr)
    throw std::runtime_error("Error in parametric_composition sampling function: mc_calculator == nullptr");
  std::vector<monte::Index> shape;
  shape.push_back(mc_calculator->system->param_composition_calculator.n_independent_compositions());
  CalculatorType* c = mc_calculator.get();
  monte::StateSamplingFunction f("param_composition", "Parametric composition", shape, [c]() -> std::vector<double> {
    if (c->param_composition_calculator == nullptr || c->param_composition_calculator->state == nullptr)
      throw std::runtime_error(
          "Error in parametric_composition sampling function: "
          "mc_calculator->param_composition_calculator->state == nullptr");
    return c->param_composition_calculator->per_unitcell();
  });
  f.device_quantity = "param_composition";
  f.device_owner = c;
  return f;
}

/// Formation energy per unit cell (basic_semigrand_canonical.hh:530-556).
template <typename CalculatorType>
monte::StateSamplingFunction make_formation_energy_f(std::shared_ptr<CalculatorType> mc_calculator) {
  if (mc_calculator == nullptr)
    throw std::runtime_error("Error in formation_energy sampling function: mc_calculator == nullptr");
  CalculatorType* c = mc_calculator.get();
  monte::StateSamplingFunction f("formation_energy", "Intensive formation energy", {}, [c]() -> std::vector<double> {
    if (c->formation_energy_calculator == nullptr || c->formation_energy_calculator->state == nullptr)
      throw std::runtime_error(
          "Error in formation_energy sampling function: mc_calculator->formation_energy_calculator->state == nullptr");
    return {c->formation_energy_calculator->per_unitcell()};
  });
  f.device_quantity = "formation_energy";
  f.device_owner = c;
  return f;
}

/// Semi-grand canonical potential energy per unit cell (basic_semigrand_canonical.hh:569-590).
template <typename CalculatorType>
monte::StateSamplingFunction make_potential_energy_f(std::shared_ptr<CalculatorType> mc_calculator) {
  if (mc_calculator == nullptr)
    throw std::runtime_error("Error in formation_energy sampling function: mc_calculator == nullptr");
  CalculatorType* c = mc_calculator.get();
  monte::StateSamplingFunction f("potential_energy", "Intensive potential energy", {}, [c]() -> std::vector<double> {
    if (c->potential.state == nullptr)
      throw std::runtime_error("Error in formation_energy sampling function: mc_calculator->potential.state == nullptr");
    return {c->potential.per_unitcell()};
  });
  f.device_quantity = "potential_energy";
  f.device_owner = c;
  return f;
}

/// The configuration as JSON text (basic_semigrand_canonical.hh:606-627).
template <typename CalculatorType>
monte::jsonStateSamplingFunction make_configuration_json_f(std::shared_ptr<CalculatorType> mc_calculator) {
  if (mc_calculator == nullptr)
    throw std::runtime_error("Error in formation_energy sampling function: mc_calculator == nullptr");
  CalculatorType* c = mc_calculator.get();
  return monte::jsonStateSamplingFunction("configuration", "Configuration values", [c]() -> std::string {
    if (c->potential.state == nullptr)
      throw std::runtime_error("Error in formation_energy sampling function: mc_calculator->potential.state == nullptr");
    return c->state->configuration.to_json();
  });
}

}  // namespace semigrand_canonical
}  // namespace ising_cpp
}  // namespace montegpu

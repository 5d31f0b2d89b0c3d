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
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "montegpu.h"

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

template <typename EngineType = std::mt19937_64>
class RandomNumberGenerator {
 public:
  explicit RandomNumberGenerator(std::shared_ptr<EngineType> _engine = nullptr) : engine(_engine) {
    if (!engine) {
      engine = std::make_shared<EngineType>();
      std::random_device device;
      engine->seed(device());
    }
  }
  template <typename IntType>
  IntType random_int(IntType maximum_value) {
    return std::uniform_int_distribution<IntType>(0, maximum_value)(*engine);
  }
  template <typename RealType>
  RealType random_real(RealType maximum_value) {
    return std::uniform_real_distribution<RealType>(0, maximum_value)(*engine);
  }
  std::shared_ptr<EngineType> engine;
};

struct OccEvent {
  std::vector<Index> linear_site_index;
  std::vector<int> new_occ;
};

class IsingConfiguration {
 public:
  IsingConfiguration() : IsingConfiguration(std::vector<int>{0, 0}, 1) {}
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

}  // namespace semigrand_canonical
}  // namespace ising_cpp
}  // namespace montegpu

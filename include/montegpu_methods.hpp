// montegpu_methods.hpp -- header-only C++ form of libcasm-monte's sampling, completion-check,
// statistics and Metropolis-method layer, with the same names, argument meaning and rules as
// the reference's C++ (namespace CASM::monte there, montegpu::monte here):
//
//   include/casm/monte/sampling/Sampler.hh:30-416          Sampler, SamplerComponent,
//                                                          RequestedPrecision, get_n_samples,
//                                                          default_component_names
//   include/casm/monte/sampling/StateSamplingFunction.hh:20-136
//                                                          StateSamplingFunction,
//                                                          jsonStateSamplingFunction
//   include/casm/monte/BasicStatistics.hh:1-120            BasicStatistics,
//                                                          BasicStatisticsCalculator
//   include/casm/monte/checks/CutoffCheck.hh:14-94         CutoffCheckParams, all_minimums_met,
//                                                          any_maximum_met
//   src/casm/monte/checks/EquilibrationCheck.cc:118-225    default_equilibration_check,
//                                                          equilibration_check
//   include/casm/monte/checks/ConvergenceCheck.hh:74-184   convergence_check
//   include/casm/monte/checks/CompletionCheck.hh:19-376    CompletionCheckParams,
//                                                          CompletionCheckResults,
//                                                          CompletionCheck
//   include/casm/monte/methods/metropolis.hh:26-35         metropolis_acceptance
//   include/casm/monte/methods/basic_occupation_metropolis.hh:18-425
//                                                          BasicOccupationMetropolisData,
//                                                          basic_occupation_metropolis
//   include/casm/monte/RandomNumberGenerator.hh:15-42      RandomNumberGenerator
//
// Eigen vectors become std::vector<double>; a Sampler keeps its samples row by row (sample
// index, then component).  JSON values (jsonStateSamplingFunction, jsonSampler) are JSON text.
// The equilibration scan and the statistics (autocorrelation-corrected precision of the mean)
// are the library's host numerics (mg_equilibration_check, mg_basic_statistics in montegpu.h),
// which equal the reference's bit for bit.  Errors throw std::runtime_error with the reference's
// messages.  The generic loop basic_occupation_metropolis runs on the host because it calls the
// caller's functions every step; the built-in models hand their passes to the GPU (see
// montegpu_ising.hpp).
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <optional>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "montegpu.h"

namespace montegpu {
namespace monte {

typedef long Index;
typedef long CountType;
typedef double TimeType;
typedef unsigned long long BigCountType;

/// Boltzmann constant (eV/K), the value of the reference's definitions.
constexpr double KB = 8.6173303e-05;

// ---------------------------------------------------------------- random numbers

/// std::uniform_int_distribution / uniform_real_distribution over a shared engine
/// (RandomNumberGenerator.hh:15-42): random_int(max) in [0, max], random_real(max) in [0, max).
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

// ---------------------------------------------------------------- run log

/// Clock of a run (the part of libcasm-global's Log the methods use): elapsed seconds since
/// restart_clock() and since begin_lap().
class Log {
 public:
  Log() { restart_clock(); }
  void restart_clock() {
    m_start = clock::now();
    m_lap = m_start;
  }
  void begin_lap() { m_lap = clock::now(); }
  double time_s() const { return std::chrono::duration<double>(clock::now() - m_start).count(); }
  double lap_time() const { return std::chrono::duration<double>(clock::now() - m_lap).count(); }

 private:
  typedef std::chrono::steady_clock clock;
  clock::time_point m_start, m_lap;
};

/// Where and how often a method writes its status (MethodLog.hh:13-38).
struct MethodLog {
  std::string logfile_path;
  std::optional<double> log_frequency;
  Log log;
  void reset() {}
};

// ---------------------------------------------------------------- samplers

inline std::vector<std::string> colmajor_component_names(Index n_rows, Index n_cols) {
  std::vector<std::string> result;
  for (Index j = 0; j < n_cols; ++j)
    for (Index i = 0; i < n_rows; ++i) result.push_back(std::to_string(i) + "," + std::to_string(j));
  return result;
}

/// Component names ["0", "1", ...] for a scalar or vector, "i,j" column-major for a matrix.
inline std::vector<std::string> default_component_names(std::vector<Index> shape) {
  if (shape.size() == 0) return {"0"};
  if (shape.size() == 1) {
    std::vector<std::string> result;
    for (Index i = 0; i < shape[0]; ++i) result.push_back(std::to_string(i));
    return result;
  }
  if (shape.size() == 2) return colmajor_component_names(shape[0], shape[1]);
  throw std::runtime_error("Error constructing sampler component names: >2 dimensions is not supported");
}

inline Index calc_n_components(std::vector<Index> const& shape) {
  Index result = 1;
  for (Index x : shape) result *= x;
  return result;
}

/// Sampled values of one quantity: one row per sample, one column per component.  Storage
/// grows by `capacity_increment` rows when full.
class Sampler {
 public:
  explicit Sampler(std::vector<Index> _shape = {}, CountType _capacity_increment = 1000)
      : m_n_components(calc_n_components(_shape)), m_component_names(default_component_names(_shape)),
        m_shape(_shape), m_capacity_increment(_capacity_increment) {
    clear();
  }
  Sampler(std::vector<Index> _shape, std::vector<std::string> const& _component_names,
          CountType _capacity_increment = 1000)
      : m_n_components(static_cast<Index>(_component_names.size())), m_component_names(_component_names),
        m_shape(_shape), m_capacity_increment(_capacity_increment) {
    clear();
  }

  void push_back(double const& value) { push_back(std::vector<double>{value}); }
  void push_back(std::vector<double> const& vector) {
    if (static_cast<Index>(vector.size()) != m_n_components)
      throw std::runtime_error("Error in Sampler::push_back: value size does not match the number of components");
    if (m_n_samples == m_capacity) set_sample_capacity(m_capacity + m_capacity_increment);
    std::copy(vector.begin(), vector.end(), m_values.begin() + m_n_samples * m_n_components);
    ++m_n_samples;
  }
  /// values[n_samples][n_components], row by row
  void set_values(std::vector<double> const& values, CountType n_samples) {
    m_values = values;
    m_n_samples = n_samples;
    m_capacity = n_samples;
  }
  void clear() {
    m_capacity = m_capacity_increment;
    m_values.assign(static_cast<size_t>(m_capacity * m_n_components), 0.0);
    m_n_samples = 0;
  }
  void set_sample_capacity(CountType sample_capacity) {
    m_values.resize(static_cast<size_t>(sample_capacity * m_n_components), 0.0);
    m_capacity = sample_capacity;
    m_n_samples = std::min(m_n_samples, sample_capacity);
  }
  void set_capacity_increment(CountType _capacity_increment) { m_capacity_increment = _capacity_increment; }
  std::vector<std::string> const& component_names() const { return m_component_names; }
  std::vector<Index> const& shape() const { return m_shape; }
  Index n_components() const { return m_n_components; }
  CountType n_samples() const { return m_n_samples; }
  CountType sample_capacity() const { return m_capacity; }
  CountType capacity_increment() const { return m_capacity_increment; }
  /// sampled values [n_samples][n_components], row by row
  std::vector<double> values() const {
    return std::vector<double>(m_values.begin(), m_values.begin() + m_n_samples * m_n_components);
  }
  /// one component over all samples
  std::vector<double> component(Index component_index) const {
    std::vector<double> out(static_cast<size_t>(m_n_samples));
    for (CountType s = 0; s < m_n_samples; ++s) out[s] = m_values[s * m_n_components + component_index];
    return out;
  }
  std::vector<double> sample(CountType sample_index) const {
    return std::vector<double>(m_values.begin() + sample_index * m_n_components,
                               m_values.begin() + (sample_index + 1) * m_n_components);
  }

 private:
  Index m_n_components;
  std::vector<std::string> m_component_names;
  std::vector<Index> m_shape;
  std::vector<double> m_values;
  CountType m_n_samples = 0;
  CountType m_capacity = 0;
  CountType m_capacity_increment;
};

typedef std::map<std::string, std::shared_ptr<Sampler>> SamplerMap;

/// Number of samples (of the first sampler; all are sampled together).
inline CountType get_n_samples(SamplerMap const& samplers) {
  if (samplers.size()) return samplers.begin()->second->n_samples();
  return CountType(0);
}

/// JSON samples, one JSON text per sample.
struct jsonSampler {
  std::vector<std::string> values;
};
typedef std::map<std::string, jsonSampler> jsonSamplerMap;

/// A sampler component requested to converge: compared by sampler name, then component index.
struct SamplerComponent {
  SamplerComponent() = default;
  SamplerComponent(std::string _sampler_name, Index _component_index, std::string _component_name)
      : sampler_name(std::move(_sampler_name)), component_index(_component_index),
        component_name(std::move(_component_name)) {}
  std::string sampler_name;
  Index component_index = 0;
  std::string component_name;
  bool operator<(SamplerComponent const& other) const {
    if (sampler_name == other.sampler_name) return component_index < other.component_index;
    return sampler_name < other.sampler_name;
  }
};

struct RequestedPrecision {
  bool abs_convergence_is_required = false;
  double abs_precision = 0.0;
  bool rel_convergence_is_required = false;
  double rel_precision = 0.0;
  static RequestedPrecision abs_and_rel(double abs_value, double rel_value) {
    RequestedPrecision x;
    x.abs_convergence_is_required = true;
    x.abs_precision = abs_value;
    x.rel_convergence_is_required = true;
    x.rel_precision = rel_value;
    return x;
  }
  static RequestedPrecision abs(double value) {
    RequestedPrecision x;
    x.abs_convergence_is_required = true;
    x.abs_precision = value;
    return x;
  }
  static RequestedPrecision rel(double value) {
    RequestedPrecision x;
    x.rel_convergence_is_required = true;
    x.rel_precision = value;
    return x;
  }
};

inline SamplerMap::const_iterator find_or_throw(SamplerMap const& samplers, SamplerComponent const& key) {
  auto it = samplers.find(key.sampler_name);
  if (it == samplers.end())
    throw std::runtime_error("Error finding sampler component: Sampler '" + key.sampler_name + "' not found.");
  if (key.component_index >= it->second->n_components())
    throw std::runtime_error("Error finding sampler component: Requested component index " +
                             std::to_string(key.component_index) + ", but '" + key.sampler_name + "' has " +
                             std::to_string(it->second->n_components()) + " components.");
  return it;
}

/// A function sampling the current state.  `device_quantity` and `device_owner` let a
/// calculator that runs its passes on the GPU take the sample from its device sums instead
/// of calling `function` on the host state (set by the built-in factories only).
struct StateSamplingFunction {
  StateSamplingFunction() = default;
  StateSamplingFunction(std::string _name, std::string _description, std::vector<Index> _shape,
                        std::function<std::vector<double>()> _function)
      : name(std::move(_name)), description(std::move(_description)), shape(_shape),
        component_names(default_component_names(_shape)), function(std::move(_function)) {}
  StateSamplingFunction(std::string _name, std::string _description,
                        std::vector<std::string> const& _component_names, std::vector<Index> _shape,
                        std::function<std::vector<double>()> _function)
      : name(std::move(_name)), description(std::move(_description)), shape(_shape),
        component_names(_component_names), function(std::move(_function)) {}
  std::string name;
  std::string description;
  std::vector<Index> shape;
  std::vector<std::string> component_names;
  std::function<std::vector<double>()> function;
  std::string device_quantity;
  const void* device_owner = nullptr;
  std::vector<double> operator()() const { return function(); }
};
typedef std::map<std::string, StateSamplingFunction> StateSamplingFunctionMap;

struct jsonStateSamplingFunction {
  jsonStateSamplingFunction() = default;
  jsonStateSamplingFunction(std::string _name, std::string _description, std::function<std::string()> _function)
      : name(std::move(_name)), description(std::move(_description)), function(std::move(_function)) {}
  std::string name;
  std::string description;
  std::function<std::string()> function;
  std::string operator()() const { return function(); }
};
typedef std::map<std::string, jsonStateSamplingFunction> jsonStateSamplingFunctionMap;

// ---------------------------------------------------------------- statistics

struct BasicStatistics {
  double mean = 0.0;
  double calculated_precision = std::numeric_limits<double>::max();
};
inline double get_calculated_precision(BasicStatistics const& stats) { return stats.calculated_precision; }
inline double get_calculated_relative_precision(BasicStatistics const& stats) {
  return std::abs(stats.calculated_precision / stats.mean);
}

/// Mean and autocorrelation-corrected precision of the mean at `confidence`
/// (BasicStatistics.cc:114-188); with sample weights, the observations are resampled at
/// `n_resamples` equally spaced points of the cumulative weight (method 1).
struct BasicStatisticsCalculator {
  explicit BasicStatisticsCalculator(double _confidence = 0.95, Index _method = 1, Index _n_resamples = 10000)
      : confidence(_confidence), method(_method), n_resamples(_n_resamples) {}
  double confidence;
  Index method;
  Index n_resamples;
  BasicStatistics operator()(std::vector<double> const& observations) const {
    return (*this)(observations, std::vector<double>());
  }
  BasicStatistics operator()(std::vector<double> const& observations, std::vector<double> const& sample_weight) const {
    BasicStatistics s;
    if (mg_basic_statistics(observations.data(), (long)observations.size(),
                            sample_weight.empty() ? nullptr : sample_weight.data(), (long)sample_weight.size(),
                            confidence, method, n_resamples, &s.mean, &s.calculated_precision) != MG_OK)
      throw std::runtime_error(mg_last_error());
    return s;
  }
};

template <typename StatisticsType>
using CalcStatisticsFunction =
    std::function<StatisticsType(std::vector<double> const& observations, std::vector<double> const& sample_weight)>;

template <typename StatisticsType>
CalcStatisticsFunction<StatisticsType> default_statistics_calculator();
template <>
inline CalcStatisticsFunction<BasicStatistics> default_statistics_calculator<BasicStatistics>() {
  return BasicStatisticsCalculator();
}

// ---------------------------------------------------------------- equilibration

struct IndividualEquilibrationCheckResult {
  bool is_equilibrated = false;
  CountType N_samples_for_equilibration = 0;
};

typedef std::function<IndividualEquilibrationCheckResult(
    std::vector<double> const& observations, std::vector<double> const& sample_weight,
    RequestedPrecision requested_precision)>
    EquilibrationCheckFunction;

/// The equilibration scan of one observable to the requested absolute precision, or to
/// |mean x relative precision| (EquilibrationCheck.cc:118-162); weighted observations are
/// w_i x_i N / W.
inline IndividualEquilibrationCheckResult default_equilibration_check(std::vector<double> const& observations,
                                                                      std::vector<double> const& sample_weight,
                                                                      RequestedPrecision requested_precision) {
  double prec;
  if (requested_precision.abs_convergence_is_required) {
    prec = requested_precision.abs_precision;
  } else if (requested_precision.rel_convergence_is_required) {
    double sum = 0.0;
    for (double v : observations) sum += v;
    const double mean = sum / static_cast<double>(observations.size());
    prec = std::abs(mean * requested_precision.rel_precision);
  } else {
    IndividualEquilibrationCheckResult result;
    result.is_equilibrated = true;
    result.N_samples_for_equilibration = 0;
    return result;
  }
  std::vector<double> obs = observations;
  if (!sample_weight.empty()) {
    if (sample_weight.size() != observations.size())
      throw std::runtime_error("Error in equilibration_check: sample_weight.size() != observations.size()");
    double W = 0.0;
    for (double w : sample_weight) W += w;
    const double weight_factor = static_cast<double>(sample_weight.size()) / W;
    for (size_t i = 0; i < obs.size(); ++i) obs[i] *= weight_factor * sample_weight[i];
  }
  int eq = 0;
  long n_eq = 0;
  if (mg_equilibration_check(obs.data(), (long)obs.size(), prec, &eq, &n_eq) != MG_OK)
    throw std::runtime_error(mg_last_error());
  IndividualEquilibrationCheckResult result;
  result.is_equilibrated = eq != 0;
  result.N_samples_for_equilibration = n_eq;
  return result;
}

struct EquilibrationCheckResults {
  bool all_equilibrated = false;
  CountType N_samples_for_all_to_equilibrate = 0;
  std::map<SamplerComponent, IndividualEquilibrationCheckResult> individual_results;
};

/// Equilibration of every requested component (EquilibrationCheck.cc:181-225); stops at the
/// first one not equilibrated unless check_all.
inline EquilibrationCheckResults equilibration_check(
    EquilibrationCheckFunction equilibration_check_f,
    std::map<SamplerComponent, RequestedPrecision> const& requested_precision, SamplerMap const& samplers,
    Sampler const& sample_weight, bool check_all) {
  if (equilibration_check_f == nullptr)
    throw std::runtime_error("Error in equilibration_check: equilibration_check_f == nullptr");
  EquilibrationCheckResults results;
  if (!requested_precision.size()) return results;
  results.all_equilibrated = true;
  const std::vector<double> weights = sample_weight.n_samples() ? sample_weight.component(0) : std::vector<double>();
  for (auto const& p : requested_precision) {
    Sampler const& sampler = *find_or_throw(samplers, p.first)->second;
    IndividualEquilibrationCheckResult current =
        equilibration_check_f(sampler.component(p.first.component_index), weights, p.second);
    results.N_samples_for_all_to_equilibrate =
        std::max(results.N_samples_for_all_to_equilibrate, current.N_samples_for_equilibration);
    results.all_equilibrated &= current.is_equilibrated;
    results.individual_results.emplace(p.first, current);
    if (!check_all && !results.all_equilibrated) break;
  }
  return results;
}

// ---------------------------------------------------------------- convergence

template <typename StatisticsType>
struct IndividualConvergenceCheckResult {
  bool is_converged = false;
  RequestedPrecision requested_precision;
  StatisticsType stats;
};

template <typename StatisticsType>
IndividualConvergenceCheckResult<StatisticsType> convergence_check(StatisticsType const& stats,
                                                                   RequestedPrecision const& requested_precision) {
  IndividualConvergenceCheckResult<StatisticsType> result;
  result.stats = stats;
  result.requested_precision = requested_precision;
  result.is_converged = true;
  if (requested_precision.abs_convergence_is_required)
    result.is_converged &= get_calculated_precision(stats) < requested_precision.abs_precision;
  if (requested_precision.rel_convergence_is_required)
    result.is_converged &= get_calculated_relative_precision(stats) < requested_precision.rel_precision;
  return result;
}

template <typename StatisticsType>
struct ConvergenceCheckResults {
  bool all_converged = false;
  CountType N_samples_for_statistics = 0;
  std::map<SamplerComponent, IndividualConvergenceCheckResult<StatisticsType>> individual_results;
};

inline std::vector<double> tail(std::vector<double> const& v, CountType n) {
  return std::vector<double>(v.end() - n, v.end());
}

/// Statistics of the last N - N_equilibration samples of each requested component
/// (ConvergenceCheck.hh:139-184).
template <typename StatisticsType>
ConvergenceCheckResults<StatisticsType> convergence_check(
    SamplerMap const& samplers, Sampler const& sample_weight,
    std::map<SamplerComponent, RequestedPrecision> const& requested_precision,
    CountType N_samples_for_equilibration, CalcStatisticsFunction<StatisticsType> calc_statistics_f) {
  ConvergenceCheckResults<StatisticsType> results;
  const CountType N_samples = get_n_samples(samplers);
  if (!requested_precision.size()) {
    results.N_samples_for_statistics = N_samples;
    return results;
  }
  if (N_samples_for_equilibration >= N_samples) return results;
  results.N_samples_for_statistics = N_samples - N_samples_for_equilibration;
  results.all_converged = true;
  if (calc_statistics_f == nullptr)
    throw std::runtime_error("Error in component_convergence_check: calc_statistics_f == nullptr");
  for (auto const& p : requested_precision) {
    Sampler const& sampler = *find_or_throw(samplers, p.first)->second;
    const std::vector<double> obs = tail(sampler.component(p.first.component_index), results.N_samples_for_statistics);
    const std::vector<double> w = sample_weight.n_samples() != 0
                                      ? tail(sample_weight.component(0), results.N_samples_for_statistics)
                                      : std::vector<double>();
    IndividualConvergenceCheckResult<StatisticsType> current = convergence_check(calc_statistics_f(obs, w), p.second);
    results.all_converged &= current.is_converged;
    results.individual_results.emplace(p.first, current);
  }
  return results;
}

// ---------------------------------------------------------------- cutoffs

struct CutoffCheckParams {
  std::optional<CountType> min_count;
  std::optional<TimeType> min_time;
  std::optional<CountType> min_sample;
  std::optional<TimeType> min_clocktime;
  std::optional<CountType> max_count;
  std::optional<TimeType> max_time;
  std::optional<CountType> max_sample;
  std::optional<TimeType> max_clocktime;
};

inline bool all_minimums_met(CutoffCheckParams const& p, std::optional<CountType> count, std::optional<TimeType> time,
                             CountType n_samples, TimeType clocktime) {
  if (p.min_sample.has_value() && n_samples < p.min_sample.value()) return false;
  if (p.min_count.has_value() && count.has_value() && count.value() < p.min_count.value()) return false;
  if (p.min_time.has_value() && time.has_value() && time.value() < p.min_time.value()) return false;
  if (p.min_clocktime.has_value() && clocktime < p.min_clocktime.value()) return false;
  return true;
}

inline bool any_maximum_met(CutoffCheckParams const& p, std::optional<CountType> count, std::optional<TimeType> time,
                            CountType n_samples, TimeType clocktime) {
  if (p.max_sample.has_value() && n_samples >= p.max_sample.value()) return true;
  if (p.max_count.has_value() && count.has_value() && count.value() >= p.max_count.value()) return true;
  if (p.max_time.has_value() && time.has_value() && time.value() >= p.max_time.value()) return true;
  if (p.max_clocktime.has_value() && clocktime >= p.max_clocktime.value()) return true;
  return false;
}

// ---------------------------------------------------------------- completion check

template <typename StatisticsType>
struct CompletionCheckParams {
  CompletionCheckParams()
      : equilibration_check_f(default_equilibration_check),
        calc_statistics_f(default_statistics_calculator<StatisticsType>()) {}
  CutoffCheckParams cutoff_params;
  EquilibrationCheckFunction equilibration_check_f;
  CalcStatisticsFunction<StatisticsType> calc_statistics_f;
  std::map<SamplerComponent, RequestedPrecision> requested_precision;
  bool log_spacing = false;
  CountType check_begin = 100;
  CountType check_period = 100;
  double check_base = 10.0;
  double check_shift = 2.0;
  CountType check_period_max = 10000;

  CountType sample_check_linear(Index n) const { return check_begin + check_period * n; }
  CountType sample_check_log(Index n) const {
    return check_begin + static_cast<CountType>(std::round(std::pow(check_base, (n + check_shift))));
  }
  Index find_n_begin_linear() const {
    Index n_begin_linear = 0;
    auto check_delta = [&](Index n) { return sample_check_log(n) - sample_check_log(n - 1); };
    while (check_delta(n_begin_linear + 1) <= check_period_max) n_begin_linear += 1;
    return n_begin_linear;
  }
  CountType sample_check_log(Index n, Index n_begin_linear) const {
    if (n <= n_begin_linear) return sample_check_log(n);
    return sample_check_log(n_begin_linear) + check_period_max * (n - n_begin_linear);
  }
};

template <typename StatisticsType>
struct CompletionCheckResults {
  CompletionCheckParams<StatisticsType> params;
  std::optional<CountType> count;
  std::optional<TimeType> time;
  TimeType clocktime = 0.0;
  CountType n_samples = 0;
  bool has_all_minimums_met = false;
  bool has_any_maximum_met = false;
  std::optional<CountType> n_samples_at_convergence_check;
  EquilibrationCheckResults equilibration_check_results;
  ConvergenceCheckResults<StatisticsType> convergence_check_results;
  bool is_complete = false;

  void partial_reset(std::optional<CountType> _count = std::nullopt, std::optional<TimeType> _time = std::nullopt,
                     TimeType _clocktime = 0.0, CountType _n_samples = 0) {
    count = _count;
    time = _time;
    clocktime = _clocktime;
    n_samples = _n_samples;
    has_all_minimums_met = false;
    has_any_maximum_met = false;
    is_complete = false;
  }
  void full_reset(std::optional<CountType> _count = std::nullopt, std::optional<TimeType> _time = std::nullopt,
                  TimeType _clocktime = 0.0, CountType _n_samples = 0) {
    partial_reset(_count, _time, _clocktime, _n_samples);
    n_samples_at_convergence_check = std::nullopt;
    equilibration_check_results = EquilibrationCheckResults();
    convergence_check_results = ConvergenceCheckResults<StatisticsType>();
  }
};

/// Cutoffs, then equilibration and convergence of the requested components on the check
/// schedule (CompletionCheck.hh:175-376).  A run calls is_complete before every step.
template <typename StatisticsType>
class CompletionCheck {
 public:
  explicit CompletionCheck(CompletionCheckParams<StatisticsType> params)
      : m_params(params), m_n_begin_linear(m_params.find_n_begin_linear()) {
    m_results.params = m_params;
    m_results.is_complete = false;
    if (m_params.equilibration_check_f == nullptr)
      throw std::runtime_error("Error constructing CompletionCheck: params.equilibration_check_f == nullptr");
    if (m_params.calc_statistics_f == nullptr)
      throw std::runtime_error("Error constructing CompletionCheck: params.calc_statistics_f == nullptr");
  }
  CompletionCheckParams<StatisticsType> const& params() const { return m_params; }
  CompletionCheckResults<StatisticsType> const& results() const { return m_results; }
  void reset() {
    m_results.full_reset();
    m_n_checks = 0;
    m_last_n_samples = 0;
    m_last_clocktime = 0.0;
  }
  bool is_complete(SamplerMap const& samplers, Sampler const& sample_weight, Log& log) {
    return _is_complete(samplers, sample_weight, std::nullopt, std::nullopt, log);
  }
  bool is_complete(SamplerMap const& samplers, Sampler const& sample_weight, CountType count, Log& log) {
    return _is_complete(samplers, sample_weight, count, std::nullopt, log);
  }
  bool is_complete(SamplerMap const& samplers, Sampler const& sample_weight, TimeType time, Log& log) {
    return _is_complete(samplers, sample_weight, std::nullopt, time, log);
  }
  bool is_complete(SamplerMap const& samplers, Sampler const& sample_weight, CountType count, TimeType time,
                   Log& log) {
    return _is_complete(samplers, sample_weight, count, time, log);
  }

  // --- used by calculators that run whole passes on the GPU: within a pass the samples and
  // the count do not change, so the calls before the pass's other steps can only advance the
  // check schedule (each re-running an identical check, whose result is the same).

  /// The effect of `n_calls` further calls with the inputs of the previous call.
  void repeat_calls(CountType n_calls) {
    CompletionCheckResults<StatisticsType> const& r = m_results;
    if (!r.has_all_minimums_met || r.has_any_maximum_met || r.is_complete) return;
    while (n_calls > 0 && r.n_samples >= check_at()) {
      m_n_checks += 1;
      n_calls -= 1;
    }
  }
  /// Whether a call with these inputs could return true or run a convergence check
  /// (clock-time minimums taken as met).
  bool could_complete_at(CountType n_samples, CountType count) const {
    CutoffCheckParams const& cp = m_params.cutoff_params;
    if (!all_minimums_met(cp, count, std::nullopt, n_samples, cp.min_clocktime.has_value() ? 1e300 : 0.0))
      return false;
    if (any_maximum_met(cp, count, std::nullopt, n_samples, 0.0)) return true;
    return n_samples >= check_at();
  }

 private:
  CountType check_at() const {
    return m_params.log_spacing ? m_params.sample_check_log(m_n_checks, m_n_begin_linear)
                                : m_params.sample_check_linear(m_n_checks);
  }
  bool _is_complete(SamplerMap const& samplers, Sampler const& sample_weight, std::optional<CountType> count,
                    std::optional<TimeType> time, Log& log) {
    const CountType n_samples = get_n_samples(samplers);
    TimeType clocktime = m_last_clocktime;
    if (n_samples != m_last_n_samples) {
      clocktime = log.time_s();
      m_last_n_samples = n_samples;
      m_last_clocktime = clocktime;
    }
    m_results.partial_reset(count, time, clocktime, n_samples);
    m_results.has_all_minimums_met = all_minimums_met(m_params.cutoff_params, count, time, n_samples, clocktime);
    if (!m_results.has_all_minimums_met) return false;
    m_results.has_any_maximum_met = any_maximum_met(m_params.cutoff_params, count, time, n_samples, clocktime);
    if (m_results.has_any_maximum_met) {
      m_results.is_complete = true;
      if (!m_results.n_samples_at_convergence_check.has_value() ||
          n_samples != m_results.n_samples_at_convergence_check.value())
        _check_convergence(samplers, sample_weight, n_samples);
      return true;
    }
    if (n_samples >= check_at()) {
      m_n_checks += 1;
      _check_convergence(samplers, sample_weight, n_samples);
    }
    if (m_results.convergence_check_results.all_converged) m_results.is_complete = true;
    return m_results.is_complete;
  }
  void _check_convergence(SamplerMap const& samplers, Sampler const& sample_weight, CountType n_samples) {
    if (m_params.requested_precision.size()) {
      m_results.n_samples_at_convergence_check = n_samples;
      m_results.equilibration_check_results = equilibration_check(
          m_params.equilibration_check_f, m_params.requested_precision, samplers, sample_weight, false);
      if (m_results.equilibration_check_results.all_equilibrated) {
        m_results.convergence_check_results = convergence_check<StatisticsType>(
            samplers, sample_weight, m_params.requested_precision,
            m_results.equilibration_check_results.N_samples_for_all_to_equilibrate, m_params.calc_statistics_f);
      } else {
        m_results.convergence_check_results = ConvergenceCheckResults<StatisticsType>();
      }
    }
  }

  CompletionCheckParams<StatisticsType> m_params;
  CompletionCheckResults<StatisticsType> m_results;
  Index m_n_checks = 0;
  Index m_n_begin_linear = 0;
  Index m_last_n_samples = 0;
  double m_last_clocktime = 0.0;
};

// ---------------------------------------------------------------- Metropolis methods

namespace methods {

/// accept if dE < 0 (no draw), else if random_real(1.0) < exp(-dE beta) (metropolis.hh:26-35)
template <typename GeneratorType>
bool metropolis_acceptance(double delta_potential_energy, double beta, GeneratorType& random_number_generator) {
  if (delta_potential_energy < 0.0) return true;
  const double rand = random_number_generator.random_real(1.0);
  const double prob = std::exp(-delta_potential_energy * beta);
  return rand < prob;
}

/// Run data and results of an occupation Metropolis run (basic_occupation_metropolis.hh:18-115).
template <typename StatisticsType>
struct BasicOccupationMetropolisData {
  typedef StatisticsType statistics_type;
  BasicOccupationMetropolisData(StateSamplingFunctionMap const& _sampling_functions,
                                jsonStateSamplingFunctionMap const& _json_sampling_functions,
                                CountType _n_steps_per_pass,
                                CompletionCheckParams<statistics_type> const& _completion_check_params)
      : sampling_functions(_sampling_functions), json_sampling_functions(_json_sampling_functions),
        sample_weight({}), n_steps_per_pass(_n_steps_per_pass), completion_check(_completion_check_params) {
    for (auto const& pair : sampling_functions)
      samplers.emplace(pair.second.name, std::make_shared<Sampler>(pair.second.shape, pair.second.component_names));
    for (auto const& pair : json_sampling_functions) json_samplers.emplace(pair.second.name, jsonSampler());
  }
  StateSamplingFunctionMap sampling_functions;
  SamplerMap samplers;
  jsonStateSamplingFunctionMap json_sampling_functions;
  jsonSamplerMap json_samplers;
  Sampler sample_weight;
  CountType n_pass = 0;
  CountType n_steps_per_pass;
  BigCountType n_accept = 0;
  BigCountType n_reject = 0;
  CompletionCheck<statistics_type> completion_check;

  double acceptance_rate() const {
    const double a = static_cast<double>(n_accept), r = static_cast<double>(n_reject);
    return a / (a + r);
  }
  double rejection_rate() const {
    const double a = static_cast<double>(n_accept), r = static_cast<double>(n_reject);
    return r / (a + r);
  }
  void reset() {
    for (auto& pair : samplers) pair.second->clear();
    for (auto& pair : json_samplers) pair.second.values.clear();
    sample_weight.clear();
    n_pass = 0;
    n_accept = 0;
    n_reject = 0;
    completion_check.reset();
  }
};

/// Write nothing; restart the log's lap timer.
template <typename StatisticsType>
void write_no_status(BasicOccupationMetropolisData<StatisticsType> const&, MethodLog& method_log) {
  method_log.log.begin_lap();
}

/// Passes, samples and speed to stdout, then the completion-check state
/// (basic_occupation_metropolis.hh:166-315).
template <typename StatisticsType>
void default_write_status(BasicOccupationMetropolisData<StatisticsType> const& data, MethodLog& method_log) {
  std::ostream& sout = std::cout;
  const double steps = static_cast<double>(data.n_pass) * static_cast<double>(data.n_steps_per_pass);
  const double time_s = method_log.log.time_s();
  sout << "Passes=" << data.n_pass << ", ";
  sout << "Samples=" << get_n_samples(data.samplers) << ", ";
  sout << "ClockTime(s)=" << time_s << ", ";
  sout << "Steps/Second=" << steps / time_s << ", ";
  sout << "Seconds/Step=" << time_s / steps << std::endl;
  auto const& results = data.completion_check.results();
  const bool all_equilibrated = results.equilibration_check_results.all_equilibrated;
  sout << "  AllEquilibrated=" << all_equilibrated << std::endl;
  if (all_equilibrated) {
    const bool all_converged = results.convergence_check_results.all_converged;
    sout << "  AllConverged=" << all_converged << std::endl;
    if (!all_converged) {
      auto const& conv = results.convergence_check_results.individual_results;
      for (auto const& pair : data.completion_check.params().requested_precision) {
        auto it = conv.find(pair.first);
        if (it == conv.end()) continue;
        const double calc_abs_prec = it->second.stats.calculated_precision;
        const double mean = it->second.stats.mean;
        const double calc_rel_prec = std::fabs(calc_abs_prec / mean);
        if (pair.second.abs_convergence_is_required)
          sout << "  - " << pair.first.sampler_name << "(" << pair.first.component_index << "): mean=" << mean
               << ", abs_prec=" << calc_abs_prec << " < requested=" << pair.second.abs_precision
               << " == " << bool(calc_abs_prec < pair.second.abs_precision) << std::endl;
        if (pair.second.rel_convergence_is_required)
          sout << "  - " << pair.first.sampler_name << "(" << pair.first.component_index << "): mean=" << mean
               << ", rel_prec=" << calc_rel_prec << " < requested=" << pair.second.rel_precision
               << " == " << bool(calc_rel_prec < pair.second.rel_precision) << std::endl;
      }
    }
  }
  method_log.reset();
  method_log.log.begin_lap();
}

/// The reference's generic occupation Metropolis loop (basic_occupation_metropolis.hh:354-425):
/// before every step the completion check; propose, potential change, Metropolis acceptance,
/// apply; n_pass advances every n_steps_per_pass steps; every sample_period passes each
/// sampling function is sampled and the status written when due.  The caller's functions run
/// every step, so this loop runs on the host; the built-in models hand whole passes to the GPU.
template <typename StatisticsType, typename EngineType, typename PotentialOccDeltaExtensiveValueF,
          typename ProposeEventF, typename ApplyEventF,
          typename WriteStatusF = void (*)(BasicOccupationMetropolisData<StatisticsType> const&, MethodLog&)>
void basic_occupation_metropolis(BasicOccupationMetropolisData<StatisticsType>& data, double temperature,
                                 PotentialOccDeltaExtensiveValueF potential_occ_delta_per_supercell_f,
                                 ProposeEventF propose_event_f, ApplyEventF apply_event_f, int sample_period = 1,
                                 std::optional<MethodLog> method_log = std::nullopt,
                                 std::shared_ptr<EngineType> random_engine = nullptr,
                                 WriteStatusF write_status_f = default_write_status<StatisticsType>) {
  const double beta = 1.0 / (KB * temperature);
  RandomNumberGenerator<EngineType> random_number_generator(random_engine);
  if (!method_log.has_value()) {
    method_log = MethodLog();
    method_log->logfile_path = "status.json";
    method_log->log_frequency = 600.0;
  }
  method_log->log.restart_clock();
  method_log->log.begin_lap();
  Index n_pass_next_sample = sample_period;
  CountType n_step = 0;
  while (!data.completion_check.is_complete(data.samplers, data.sample_weight, data.n_pass, method_log->log)) {
    auto const& event = propose_event_f(random_number_generator);
    const double delta_potential_energy = potential_occ_delta_per_supercell_f(event);
    if (metropolis_acceptance(delta_potential_energy, beta, random_number_generator)) {
      data.n_accept++;
      apply_event_f(event);
    } else {
      data.n_reject++;
    }
    n_step++;
    if (n_step == data.n_steps_per_pass) {
      n_step = 0;
      data.n_pass += 1;
    }
    if (data.n_pass == n_pass_next_sample) {
      n_pass_next_sample += sample_period;
      for (auto const& pair : data.sampling_functions) data.samplers.at(pair.second.name)->push_back(pair.second());
      for (auto const& pair : data.json_sampling_functions)
        data.json_samplers.at(pair.second.name).values.push_back(pair.second());
      if (method_log->log_frequency.has_value() && method_log->log.lap_time() >= method_log->log_frequency.value())
        write_status_f(data, *method_log);
    }
  }
  write_status_f(data, *method_log);
}

}  // namespace methods
}  // namespace monte
}  // namespace montegpu

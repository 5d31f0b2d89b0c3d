// ORACLE (test infrastructure only): CPU restatement of libcasm-monte's sampling,
// completion-check, equilibration, convergence and statistics layer.  Used only by
// tests/, __graft_entry__.smoke() and bench.py's CPU baseline, as the checker.
//
// Restates, in plain C++17 without Eigen:
//   include/casm/monte/misc/math.hh:10-72            covariance/variance/approx_erf_inv
//   src/casm/monte/BasicStatistics.cc:24-188         autocorrelation_factor, resample,
//                                                    BasicStatisticsCalculator
//   src/casm/monte/checks/EquilibrationCheck.cc:50-225
//   include/casm/monte/checks/ConvergenceCheck.hh:74-184
//   include/casm/monte/checks/CutoffCheck.hh:14-94
//   include/casm/monte/checks/CompletionCheck.hh:19-376
//   include/casm/monte/sampling/Sampler.hh (row-per-sample store, get_n_samples)
#pragma once
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <map>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

namespace oracle {

typedef long CountType;

// ---- misc/math.hh:10-72 ----
inline double mean_of(const double* x, long n) {
  // Eigen's VectorXd::mean() = sum()/size(); sum() is a redux whose association order
  // for vectorised builds differs; the oracle uses a left-to-right sum.
  double s = 0.0;
  for (long i = 0; i < n; ++i) s += x[i];
  return s / n;
}
inline double covariance_m(const double* x, const double* y, long n, double mean) {
  double cov = 0.0;
  for (long i = 0; i < n; ++i) cov += (x[i] - mean) * (y[i] - mean);
  return cov / n;
}
inline double variance_m(const double* x, long n, double mean) {
  double cov = 0.0;
  for (long i = 0; i < n; ++i) {
    double d = x[i] - mean;
    cov += d * d;
  }
  return cov / n;
}
inline double weighted_variance(const double* x, long n, double mean, const double* w,
                                double wsum) {
  double cov = 0.0;
  for (long i = 0; i < n; ++i) {
    double d = x[i] - mean;
    cov += w[i] * d * d;
  }
  return cov / wsum;
}
// Winitzki's approximation, a = 0.147 (math.hh:62-72)
inline double approx_erf_inv(double x) {
  const double one = 1.0;
  const double PI = 3.141592653589793238463;
  const double a = 0.147;
  double sgn = (x < 0.0) ? -one : one;
  double b = std::log((one - x) * (one + x));
  double c = 2.0 / (PI * a) + b * 0.5;
  double d = b / a;
  return sgn * std::sqrt(std::sqrt(c * c - d) - c);
}

// ---- BasicStatistics.cc:24-48 ----
inline double autocorrelation_factor(const double* x, long N, double increment = 1.0) {
  double mean = mean_of(x, N);
  double CoVar0 = variance_m(x, N, mean);
  if (std::abs(CoVar0 / mean) < 1e-8 || CoVar0 == 0.0) return 1.0;
  for (long i = 1; i < N; ++i) {
    long range_size = N - i;
    double cov = covariance_m(x, x + i, range_size, mean);
    if (std::abs(cov / CoVar0) <= 0.5) {
      double rho = std::pow(2.0, (-1.0 / (i * increment)));
      return (1.0 + rho) / (1.0 - rho);
    }
  }
  return std::numeric_limits<double>::max();
}

// BasicStatistics.cc:50-71
inline std::vector<double> resample(const double* obs, const double* w, long n,
                                    double wsum, long n_equally_spaced) {
  (void)n;
  double increment = wsum / n_equally_spaced;
  std::vector<double> out(n_equally_spaced);
  long j = 0;
  double W_j = 0.0;
  for (long i = 0; i < n_equally_spaced; ++i) {
    double W_target = i * increment;
    while (W_j + w[j] < W_target) {
      W_j += w[j];
      ++j;
    }
    out[i] = obs[j];
  }
  return out;
}

struct BasicStatistics {
  double mean = 0.0;
  double calculated_precision = std::numeric_limits<double>::max();
};

// BasicStatistics.cc:114-188
struct BasicStatisticsCalculator {
  double confidence = 0.95;
  long method = 1;
  long n_resamples = 10000;

  BasicStatistics operator()(const double* x, long N) const {
    if (N == 0) throw std::runtime_error("Error in BasicStatisticsCalculator: observations.size()==0");
    BasicStatistics s;
    s.mean = mean_of(x, N);
    double CoVar0 = variance_m(x, N, s.mean);
    double f_autocorr = autocorrelation_factor(x, N);
    double f_confidence = std::sqrt(2.0) * approx_erf_inv(confidence);
    s.calculated_precision = f_confidence * std::sqrt(f_autocorr * CoVar0 / N);
    return s;
  }
  BasicStatistics operator()(const double* x, long N, const double* w, long nw) const {
    if (N == 0) throw std::runtime_error("Error in BasicStatisticsCalculator: observations.size()==0");
    if (nw == 0) return (*this)(x, N);
    if (nw != N) throw std::runtime_error("Error in BasicStatisticsCalculator: size mismatch");
    double W = 0.0;
    for (long i = 0; i < N; ++i) W += w[i];
    double increment = W / n_resamples;
    std::vector<double> eq = resample(x, w, N, W, n_resamples);
    if (method == 1) {
      BasicStatistics s;
      double dot = 0.0;
      for (long i = 0; i < N; ++i) dot += x[i] * w[i];
      s.mean = dot / W;
      double wvar = weighted_variance(x, N, s.mean, w, W);
      double f_autocorr = autocorrelation_factor(eq.data(), (long)eq.size(), increment);
      double f_confidence = std::sqrt(2.0) * approx_erf_inv(confidence);
      s.calculated_precision = f_confidence * std::sqrt(f_autocorr * wvar / W);
      return s;
    } else if (method == 2) {
      return (*this)(eq.data(), (long)eq.size());
    }
    throw std::runtime_error("Error in BasicStatisticsCalculator: invalid method");
  }
};

struct RequestedPrecision {
  bool abs_convergence_is_required = false;
  double abs_precision = 0.0;
  bool rel_convergence_is_required = false;
  double rel_precision = 0.0;
};

struct EquilibrationResult {
  bool is_equilibrated = false;
  CountType N_samples_for_equilibration = 0;
};

// EquilibrationCheck.cc:50-117
inline EquilibrationResult default_equilibration_check_raw(const double* obs, long N, double prec) {
  if (N == 0) throw std::runtime_error("Error in equilibration_check: observations.size()==0");
  EquilibrationResult result;
  double eps = (obs[0] == 0.0) ? 1e-8 : std::abs(obs[0]) * 1e-8;
  bool is_even = ((N % 2) == 0);
  bool all_same = true;
  for (long i = 0; i < N; i++)
    if (std::abs(obs[i] - obs[0]) > eps) {
      all_same = false;
      break;
    }
  if (all_same) {
    result.is_equilibrated = true;
    result.N_samples_for_equilibration = 0;
    return result;
  }
  long start1 = 0;
  long start2 = is_even ? N / 2 : (N / 2) + 1;
  double sum1 = 0.0, sum2 = 0.0;
  for (long i = 0; i < start2; ++i) sum1 += obs[i];
  for (long i = start2; i < N; ++i) sum2 += obs[i];
  while (std::abs((sum1 / (start2 - start1)) - (sum2 / (N - start2))) > prec && start1 < N - 2) {
    if (is_even) {
      sum1 -= obs[start1];
      sum1 += obs[start2];
      sum2 -= obs[start2];
      start2++;
    } else {
      sum1 -= obs[start1];
    }
    start1++;
    is_even = !is_even;
  }
  double mean_tot = (sum1 + sum2) / (N - start1);
  if (obs[start1] < mean_tot) {
    while (obs[start1] < mean_tot && start1 < N - 1) start1++;
  } else {
    while (obs[start1] > mean_tot && start1 < N - 1) start1++;
  }
  result.is_equilibrated = (start1 < N - 1);
  result.N_samples_for_equilibration = start1;
  return result;
}

// EquilibrationCheck.cc:119-162
inline EquilibrationResult default_equilibration_check(const double* obs, long N, const double* w,
                                                       long nw, const RequestedPrecision& req) {
  double prec;
  if (req.abs_convergence_is_required) {
    prec = req.abs_precision;
  } else if (req.rel_convergence_is_required) {
    prec = std::abs(mean_of(obs, N) * req.rel_precision);
  } else {
    EquilibrationResult r;
    r.is_equilibrated = true;
    r.N_samples_for_equilibration = 0;
    return r;
  }
  if (nw == 0) return default_equilibration_check_raw(obs, N, prec);
  if (nw != N) throw std::runtime_error("Error in equilibration_check: sample_weight.size() != observations.size()");
  double W = 0.0;
  for (long i = 0; i < nw; ++i) W += w[i];
  double weight_factor = N / W;
  std::vector<double> wo(obs, obs + N);
  for (long i = 0; i < N; ++i) wo[i] *= weight_factor * w[i];
  return default_equilibration_check_raw(wo.data(), N, prec);
}

// A sampler: n_components columns, stored component-major for convenience.
struct Sampler {
  long n_components = 1;
  std::vector<std::vector<double>> cols;  // cols[c][sample]
  explicit Sampler(long nc = 1) : n_components(nc), cols(nc) {}
  long n_samples() const { return cols.empty() ? 0 : (long)cols[0].size(); }
  void push_back(const std::vector<double>& v) {
    for (long c = 0; c < n_components; ++c) cols[c].push_back(v[c]);
  }
};

struct SamplerComponent {
  std::string sampler_name;
  long component_index = 0;
  bool operator<(const SamplerComponent& o) const {
    if (sampler_name == o.sampler_name) return component_index < o.component_index;
    return sampler_name < o.sampler_name;
  }
};

typedef std::map<std::string, Sampler> SamplerMap;

inline CountType get_n_samples(const SamplerMap& s) {
  if (s.size()) return s.begin()->second.n_samples();
  return 0;
}

struct EquilibrationCheckResults {
  bool all_equilibrated = false;
  CountType N_samples_for_all_to_equilibrate = 0;
  std::map<SamplerComponent, EquilibrationResult> individual_results;
};

struct IndividualConvergenceResult {
  bool is_converged = false;
  RequestedPrecision requested_precision;
  BasicStatistics stats;
};

struct ConvergenceCheckResults {
  bool all_converged = false;
  CountType N_samples_for_statistics = 0;
  std::map<SamplerComponent, IndividualConvergenceResult> individual_results;
};

// CutoffCheck.hh:14-94
struct CutoffCheckParams {
  std::optional<CountType> min_count, min_sample, max_count, max_sample;
  std::optional<double> min_time, min_clocktime, max_time, max_clocktime;
};

inline bool all_minimums_met(const CutoffCheckParams& p, std::optional<CountType> count,
                             std::optional<double> time, CountType n_samples, double clocktime) {
  if (p.min_sample.has_value() && n_samples < p.min_sample.value()) return false;
  if (p.min_count.has_value() && count.has_value() && count.value() < p.min_count.value()) return false;
  if (p.min_time.has_value() && time.has_value() && time.value() < p.min_time.value()) return false;
  if (p.min_clocktime.has_value() && clocktime < p.min_clocktime.value()) return false;
  return true;
}
inline bool any_maximum_met(const CutoffCheckParams& p, std::optional<CountType> count,
                            std::optional<double> time, CountType n_samples, double clocktime) {
  if (p.max_sample.has_value() && n_samples >= p.max_sample.value()) return true;
  if (p.max_count.has_value() && count.has_value() && count.value() >= p.max_count.value()) return true;
  if (p.max_time.has_value() && time.has_value() && time.value() >= p.max_time.value()) return true;
  if (p.max_clocktime.has_value() && clocktime >= p.max_clocktime.value()) return true;
  return false;
}

// CompletionCheck.hh:19-100
struct CompletionCheckParams {
  CutoffCheckParams cutoff_params;
  BasicStatisticsCalculator calc_statistics;
  std::map<SamplerComponent, RequestedPrecision> requested_precision;
  bool log_spacing = false;
  CountType check_begin = 100;
  CountType check_period = 100;
  double check_base = 10.0;
  double check_shift = 2.0;
  CountType check_period_max = 10000;

  CountType sample_check_linear(long n) const { return check_begin + check_period * n; }
  CountType sample_check_log(long n) const {
    return check_begin + static_cast<CountType>(std::round(std::pow(check_base, (n + check_shift))));
  }
  long find_n_begin_linear() const {
    long n = 0;
    auto delta = [&](long k) { return sample_check_log(k) - sample_check_log(k - 1); };
    while (delta(n + 1) <= check_period_max) n += 1;
    return n;
  }
  CountType sample_check_log(long n, long n_begin_linear) const {
    if (n <= n_begin_linear) return sample_check_log(n);
    return sample_check_log(n_begin_linear) + check_period_max * (n - n_begin_linear);
  }
};

struct CompletionCheckResults {
  std::optional<CountType> count;
  std::optional<double> time;
  double clocktime = 0.0;
  CountType n_samples = 0;
  bool has_all_minimums_met = false;
  bool has_any_maximum_met = false;
  std::optional<CountType> n_samples_at_convergence_check;
  EquilibrationCheckResults equilibration_check_results;
  ConvergenceCheckResults convergence_check_results;
  bool is_complete = false;
};

// EquilibrationCheck.cc:180-225 (check_all=false: stop at the first failure)
inline EquilibrationCheckResults equilibration_check(
    const std::map<SamplerComponent, RequestedPrecision>& req, const SamplerMap& samplers,
    const Sampler& sample_weight, bool check_all) {
  EquilibrationCheckResults results;
  if (!req.size()) return results;
  results.all_equilibrated = true;
  const double* w = sample_weight.n_samples() ? sample_weight.cols[0].data() : nullptr;
  long nw = sample_weight.n_samples();
  for (auto const& p : req) {
    auto it = samplers.find(p.first.sampler_name);
    if (it == samplers.end()) throw std::runtime_error("Error finding sampler component: Sampler '" + p.first.sampler_name + "' not found.");
    const auto& col = it->second.cols.at(p.first.component_index);
    EquilibrationResult cur = default_equilibration_check(col.data(), (long)col.size(), w, nw, p.second);
    results.N_samples_for_all_to_equilibrate =
        std::max(results.N_samples_for_all_to_equilibrate, cur.N_samples_for_equilibration);
    results.all_equilibrated &= cur.is_equilibrated;
    results.individual_results.emplace(p.first, cur);
    if (!check_all && !results.all_equilibrated) break;
  }
  return results;
}

// ConvergenceCheck.hh:74-184
inline ConvergenceCheckResults convergence_check(
    const SamplerMap& samplers, const Sampler& sample_weight,
    const std::map<SamplerComponent, RequestedPrecision>& req, CountType N_eq,
    const BasicStatisticsCalculator& calc) {
  ConvergenceCheckResults results;
  CountType N_samples = get_n_samples(samplers);
  if (!req.size()) {
    results.N_samples_for_statistics = N_samples;
    return results;
  }
  if (N_eq >= N_samples) return results;
  results.N_samples_for_statistics = N_samples - N_eq;
  results.all_converged = true;
  long n = results.N_samples_for_statistics;
  for (auto const& p : req) {
    auto it = samplers.find(p.first.sampler_name);
    const auto& col = it->second.cols.at(p.first.component_index);
    const double* tail = col.data() + (col.size() - n);
    BasicStatistics st;
    if (sample_weight.n_samples() != 0) {
      const auto& wc = sample_weight.cols[0];
      st = calc(tail, n, wc.data() + (wc.size() - n), n);
    } else {
      st = calc(tail, n);
    }
    IndividualConvergenceResult cur;
    cur.stats = st;
    cur.requested_precision = p.second;
    cur.is_converged = true;
    if (p.second.abs_convergence_is_required)
      cur.is_converged &= st.calculated_precision < p.second.abs_precision;
    if (p.second.rel_convergence_is_required)
      cur.is_converged &= std::abs(st.calculated_precision / st.mean) < p.second.rel_precision;
    results.all_converged &= cur.is_converged;
    results.individual_results.emplace(p.first, cur);
  }
  return results;
}

// CompletionCheck.hh:175-376
class CompletionCheck {
 public:
  explicit CompletionCheck(const CompletionCheckParams& p)
      : m_params(p), m_n_begin_linear(p.find_n_begin_linear()) {}
  const CompletionCheckResults& results() const { return m_results; }
  long n_checks() const { return m_n_checks; }

  bool is_complete(const SamplerMap& samplers, const Sampler& sample_weight,
                   std::optional<CountType> count, std::optional<double> time, double clocktime_now) {
    CountType n_samples = get_n_samples(samplers);
    double clocktime = m_last_clocktime;
    if (n_samples != m_last_n_samples) {
      clocktime = clocktime_now;
      m_last_n_samples = n_samples;
      m_last_clocktime = clocktime;
    }
    // partial_reset
    m_results.count = count;
    m_results.time = time;
    m_results.clocktime = clocktime;
    m_results.n_samples = n_samples;
    m_results.has_all_minimums_met = false;
    m_results.has_any_maximum_met = false;
    m_results.is_complete = false;

    m_results.has_all_minimums_met = all_minimums_met(m_params.cutoff_params, count, time, n_samples, clocktime);
    if (!m_results.has_all_minimums_met) return false;
    m_results.has_any_maximum_met = any_maximum_met(m_params.cutoff_params, count, time, n_samples, clocktime);
    if (m_results.has_any_maximum_met) {
      m_results.is_complete = true;
      if (!m_results.n_samples_at_convergence_check.has_value() ||
          n_samples != m_results.n_samples_at_convergence_check.value()) {
        check_convergence(samplers, sample_weight, n_samples);
      }
      return true;
    }
    long check_at = m_params.log_spacing ? m_params.sample_check_log(m_n_checks, m_n_begin_linear)
                                         : m_params.sample_check_linear(m_n_checks);
    if (n_samples >= check_at) {
      m_n_checks += 1;
      check_convergence(samplers, sample_weight, n_samples);
    }
    if (m_results.convergence_check_results.all_converged) m_results.is_complete = true;
    return m_results.is_complete;
  }

 private:
  void check_convergence(const SamplerMap& samplers, const Sampler& sample_weight, CountType n_samples) {
    if (m_params.requested_precision.size()) {
      m_results.n_samples_at_convergence_check = n_samples;
      m_results.equilibration_check_results =
          equilibration_check(m_params.requested_precision, samplers, sample_weight, false);
      if (m_results.equilibration_check_results.all_equilibrated) {
        m_results.convergence_check_results = convergence_check(
            samplers, sample_weight, m_params.requested_precision,
            m_results.equilibration_check_results.N_samples_for_all_to_equilibrate,
            m_params.calc_statistics);
      } else {
        m_results.convergence_check_results = ConvergenceCheckResults();
      }
    }
  }
  CompletionCheckParams m_params;
  CompletionCheckResults m_results;
  long m_n_checks = 0;
  long m_n_begin_linear = 0;
  long m_last_n_samples = 0;
  double m_last_clocktime = 0.0;
};

}  // namespace oracle

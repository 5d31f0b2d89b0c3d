// Library-level C-ABI: errors, device queries, the mt19937_64 engine, statistics.
#include <cuda_runtime.h>

#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/montegpu.h"
#include "mg_common.cuh"
#include "stats.cuh"

namespace mg {

namespace {
thread_local std::string g_error;
}

void set_error(const std::string& msg) { g_error = msg; }
const char* last_error() { return g_error.c_str(); }

}  // namespace mg

struct mg_engine {
  std::mt19937_64 e;
};

extern "C" {

const char* mg_last_error(void) { return mg::last_error(); }

int mg_version(void) { return 100; }

int mg_device_count(int* n) {
  if (!n) {
    mg::set_error("Error in mg_device_count: null pointer");
    return MG_ERR_INVALID;
  }
  MG_CUDA_TRY(cudaGetDeviceCount(n));
  return MG_OK;
}

int mg_device_sm_count(int* n) {
  if (!n) {
    mg::set_error("Error in mg_device_sm_count: null pointer");
    return MG_ERR_INVALID;
  }
  int dev = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(n, cudaDevAttrMultiProcessorCount, dev));
  return MG_OK;
}

// ---- engine (RandomNumberGenerator.hh:15-42; monte.cpp:469-545) ----
int mg_engine_create(int seed_from_device, mg_engine** out) {
  if (!out) {
    mg::set_error("Error in mg_engine_create: null pointer");
    return MG_ERR_INVALID;
  }
  auto* h = new mg_engine();
  if (seed_from_device) {
    std::random_device device;
    h->e.seed(device());
  }
  *out = h;
  return MG_OK;
}

int mg_engine_destroy(mg_engine* e) {
  delete e;
  return MG_OK;
}

int mg_engine_seed(mg_engine* e, uint64_t value) {
  if (!e) {
    mg::set_error("Error in mg_engine_seed: null engine");
    return MG_ERR_INVALID;
  }
  e->e.seed(value);
  return MG_OK;
}

int mg_engine_seed_seq(mg_engine* e, const uint64_t* values, size_t n) {
  if (!e || (n && !values)) {
    mg::set_error("Error in mg_engine_seed_seq: invalid argument");
    return MG_ERR_INVALID;
  }
  std::vector<uint64_t> v(values, values + n);
  std::seed_seq ss(v.begin(), v.end());
  e->e.seed(ss);
  return MG_OK;
}

int mg_engine_dump(const mg_engine* e, char* buf, size_t len) {
  if (!e || !buf) {
    mg::set_error("Error in mg_engine_dump: invalid argument");
    return MG_ERR_INVALID;
  }
  std::stringstream ss;
  ss << e->e;
  const std::string s = ss.str();
  if (s.size() + 1 > len) {
    mg::set_error("Error in mg_engine_dump: buffer too small");
    return MG_ERR_INVALID;
  }
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return MG_OK;
}

int mg_engine_load(mg_engine* e, const char* state) {
  if (!e || !state) {
    mg::set_error("Error in mg_engine_load: invalid argument");
    return MG_ERR_INVALID;
  }
  std::stringstream ss(state);
  std::mt19937_64 tmp;
  ss >> tmp;
  if (ss.fail()) {
    mg::set_error("Error in mg_engine_load: malformed engine state");
    return MG_ERR_INVALID;
  }
  e->e = tmp;
  return MG_OK;
}

int mg_engine_random_int(mg_engine* e, uint64_t max, uint64_t* out) {
  if (!e || !out) {
    mg::set_error("Error in mg_engine_random_int: invalid argument");
    return MG_ERR_INVALID;
  }
  *out = std::uniform_int_distribution<uint64_t>(0, max)(e->e);
  return MG_OK;
}

int mg_engine_random_real(mg_engine* e, double max, double* out) {
  if (!e || !out) {
    mg::set_error("Error in mg_engine_random_real: invalid argument");
    return MG_ERR_INVALID;
  }
  *out = std::uniform_real_distribution<double>(0, max)(e->e);
  return MG_OK;
}

// ---- statistics ----
int mg_equilibration_check(const double* obs, long n, double prec, int* is_equilibrated,
                           long* n_samples_for_equilibration) {
  if (!obs || n <= 0 || !is_equilibrated || !n_samples_for_equilibration) {
    mg::set_error("Error in equilibration_check: observations.size()==0");
    return MG_ERR_INVALID;
  }
  const mg::stats::Equilibration r = mg::stats::equilibration_check(obs, n, prec);
  *is_equilibrated = r.equilibrated ? 1 : 0;
  *n_samples_for_equilibration = r.n_equilibration;
  return MG_OK;
}

int mg_autocorrelation_factor(const double* obs, long n, double increment, double* out) {
  if (!obs || n <= 0 || !out) {
    mg::set_error("Error in autocorrelation_factor: invalid argument");
    return MG_ERR_INVALID;
  }
  *out = mg::stats::autocorrelation(obs, n, increment);
  return MG_OK;
}

double mg_approx_erf_inv(double x) { return mg::stats::erf_inv_winitzki(x); }

// BasicStatisticsCalculator::operator() (BasicStatistics.cc:114-188), weighted variants
// resample the weighted series at n_resamples equally spaced weight points.
int mg_basic_statistics(const double* obs, long n, const double* w, long nw, double confidence,
                        long method, long n_resamples, double* mean, double* calculated_precision) {
  if (!obs || n <= 0 || !mean || !calculated_precision) {
    mg::set_error("Error in BasicStatisticsCalculator: observations.size()==0");
    return MG_ERR_INVALID;
  }
  if (nw == 0) {
    const mg::stats::MeanPrecision r = mg::stats::basic_statistics(obs, n, confidence);
    *mean = r.mean;
    *calculated_precision = r.precision;
    return MG_OK;
  }
  if (nw != n || !w) {
    mg::set_error("Error in BasicStatisticsCalculator: observations.size() != sample_weight.size()");
    return MG_ERR_INVALID;
  }
  if (n_resamples <= 0) {
    mg::set_error("Error in BasicStatisticsCalculator: n_resamples must be > 0");
    return MG_ERR_INVALID;
  }
  double W = 0.0;
  for (long i = 0; i < n; ++i) W += w[i];
  const double increment = W / n_resamples;
  std::vector<double> eq(n_resamples);
  long j = 0;
  double Wj = 0.0;
  for (long i = 0; i < n_resamples; ++i) {
    const double target = i * increment;
    while (Wj + w[j] < target) {
      Wj += w[j];
      ++j;
    }
    eq[i] = obs[j];
  }
  if (method == 1) {
    double dot = 0.0;
    for (long i = 0; i < n; ++i) dot += obs[i] * w[i];
    const double m = dot / W;
    double wv = 0.0;
    for (long i = 0; i < n; ++i) {
      const double d = obs[i] - m;
      wv += w[i] * d * d;
    }
    wv /= W;
    const double f = mg::stats::autocorrelation(eq.data(), n_resamples, increment);
    const double z = sqrt(2.0) * mg::stats::erf_inv_winitzki(confidence);
    *mean = m;
    *calculated_precision = z * sqrt(f * wv / W);
    return MG_OK;
  }
  if (method == 2) {
    const mg::stats::MeanPrecision r = mg::stats::basic_statistics(eq.data(), n_resamples, confidence);
    *mean = r.mean;
    *calculated_precision = r.precision;
    return MG_OK;
  }
  mg::set_error("Error in BasicStatisticsCalculator: invalid method");
  return MG_ERR_INVALID;
}

}  // extern "C"

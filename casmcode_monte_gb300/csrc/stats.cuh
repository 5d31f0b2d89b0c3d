// Equilibration and statistics numerics of the reference's completion check, written
// once for host and device (the serving loop runs the same code per chain on the GPU).
//
//   equilibration_check  <- src/casm/monte/checks/EquilibrationCheck.cc:50-117
//                           (Van de Walle & Asta, MSMSE 10 (2002) 521: two-half mean
//                           test with advancing start, then cross the total mean)
//   autocorrelation      <- src/casm/monte/BasicStatistics.cc:24-48
//   basic_statistics     <- src/casm/monte/BasicStatistics.cc:114-131
//   approx_erf_inv       <- include/casm/monte/misc/math.hh:62-72 (Winitzki, a = 0.147)
// Sums run left to right (the reference's Eigen reductions may associate differently
// when vectorised; results agree to rounding).
#pragma once
#include <cfloat>
#include <cmath>

namespace mg {
namespace stats {

#ifdef __CUDACC__
#define MG_HD __host__ __device__
#else
#define MG_HD
#endif

MG_HD inline double series_mean(const double* x, long n) {
  double s = 0.0;
  for (long i = 0; i < n; ++i) s += x[i];
  return s / n;
}

MG_HD inline double series_variance(const double* x, long n, double m) {
  double acc = 0.0;
  for (long i = 0; i < n; ++i) {
    const double d = x[i] - m;
    acc += d * d;
  }
  return acc / n;
}

MG_HD inline double lag_covariance(const double* x, long n, long lag, double m) {
  const long len = n - lag;
  double acc = 0.0;
  for (long i = 0; i < len; ++i) acc += (x[i] - m) * (x[i + lag] - m);
  return acc / len;
}

MG_HD inline double erf_inv_winitzki(double x) {
  const double a = 0.147;
  const double pi = 3.141592653589793238463;
  const double sgn = (x < 0.0) ? -1.0 : 1.0;
  const double b = log((1.0 - x) * (1.0 + x));
  const double c = 2.0 / (pi * a) + b * 0.5;
  const double d = b / a;
  return sgn * sqrt(sqrt(c * c - d) - c);
}

// (1 + rho) / (1 - rho) with rho = 2^(-1/(k* increment)), k* the first lag whose
// autocovariance is at most half the variance; DBL_MAX if none, 1 if no variation.
MG_HD inline double autocorrelation(const double* x, long n, double increment) {
  const double m = series_mean(x, n);
  const double v0 = series_variance(x, n, m);
  if (fabs(v0 / m) < 1e-8 || v0 == 0.0) return 1.0;
  for (long k = 1; k < n; ++k) {
    const double cov = lag_covariance(x, n, k, m);
    if (fabs(cov / v0) <= 0.5) {
      const double rho = pow(2.0, (-1.0 / (k * increment)));
      return (1.0 + rho) / (1.0 - rho);
    }
  }
  return DBL_MAX;
}

struct MeanPrecision {
  double mean;
  double precision;
};

MG_HD inline MeanPrecision basic_statistics(const double* x, long n, double confidence) {
  MeanPrecision r;
  r.mean = series_mean(x, n);
  const double v0 = series_variance(x, n, r.mean);
  const double f = autocorrelation(x, n, 1.0);
  const double z = sqrt(2.0) * erf_inv_winitzki(confidence);
  r.precision = z * sqrt(f * v0 / n);
  return r;
}

struct Equilibration {
  bool equilibrated;
  long n_equilibration;
};

MG_HD inline Equilibration equilibration_check(const double* x, long n, double prec) {
  Equilibration r;
  const double x0 = x[0];
  const double tol = (x0 == 0.0) ? 1e-8 : fabs(x0) * 1e-8;
  bool flat = true;
  for (long i = 0; i < n; ++i)
    if (fabs(x[i] - x0) > tol) {
      flat = false;
      break;
    }
  if (flat) {
    r.equilibrated = true;
    r.n_equilibration = 0;
    return r;
  }
  bool even = (n % 2) == 0;
  long a = 0;                            // start of the first partition
  long b = even ? n / 2 : n / 2 + 1;     // start of the second partition
  double s1 = 0.0, s2 = 0.0;
  for (long i = 0; i < b; ++i) s1 += x[i];
  for (long i = b; i < n; ++i) s2 += x[i];
  while (fabs((s1 / (b - a)) - (s2 / (n - b))) > prec && a < n - 2) {
    if (even) {
      s1 -= x[a];
      s1 += x[b];
      s2 -= x[b];
      ++b;
    } else {
      s1 -= x[a];
    }
    ++a;
    even = !even;
  }
  const double mean_all = (s1 + s2) / (n - a);
  if (x[a] < mean_all) {
    while (x[a] < mean_all && a < n - 1) ++a;
  } else {
    while (x[a] > mean_all && a < n - 1) ++a;
  }
  r.equilibrated = a < n - 1;
  r.n_equilibration = a;
  return r;
}

}  // namespace stats
}  // namespace mg

// ORACLE (test infrastructure only): CPU restatement of the 2-D Ising semi-grand
// canonical Metropolis path of libcasm-monte, run exactly as the reference runs it.
//
// Restates:
//   include/casm/monte/ising_cpp/model.hh:19-452      IsingConfiguration, IsingFormationEnergy
//                                                    (both use_nlist branches),
//                                                    IsingParamComposition
//   include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:104-199, 268-321, 416-470
//   include/casm/monte/methods/basic_occupation_metropolis.hh:354-425
//   include/casm/monte/methods/metropolis.hh:26-35
//   include/casm/monte/RandomNumberGenerator.hh:15-42 with definitions.hh:17
//     (std::mt19937_64 and the libstdc++ uniform distributions, called exactly as there)
// KB is CASM's Boltzmann constant in eV/K as defined by libcasm-global (8.6173303e-05).
#pragma once
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "oracle_stats.hh"

namespace oracle {

constexpr double KB = 8.6173303E-05;

// RandomNumberGenerator.hh:32-41
struct RNG {
  std::mt19937_64* engine;
  long random_int(long max) { return std::uniform_int_distribution<long>(0, max)(*engine); }
  double random_real(double max) { return std::uniform_real_distribution<double>(0, max)(*engine); }
};

// metropolis.hh:26-35
inline bool metropolis_acceptance(double dE, double beta, RNG& rng) {
  if (dE < 0.0) return true;
  double rand = rng.random_real(1.0);
  double prob = std::exp(-dE * beta);
  return rand < prob;
}

struct IsingModel {
  long rows, cols;  // shape[0], shape[1]
  double J;
  bool use_nlist;
  std::vector<int> occ;  // column-major: l = rows*j + i
  std::vector<long> nlist;   // 2 per site
  std::vector<long> flower;  // 4 per site

  long n() const { return rows * cols; }
  long within(long index, int dim) const {
    long s = dim == 0 ? rows : cols;
    long r = index % s;
    if (r < 0) r += s;
    return r;
  }
  long lin(long i, long j) const { return rows * j + i; }

  // model.hh:210-256
  void build_nlist() {
    nlist.assign(2 * n(), 0);
    flower.assign(4 * n(), 0);
    for (long l = 0; l < n(); ++l) {
      long i = l % rows, j = l / rows;
      nlist[2 * l + 0] = lin(within(i + 1, 0), j);
      nlist[2 * l + 1] = lin(i, within(j + 1, 1));
      flower[4 * l + 0] = lin(within(i + 1, 0), j);
      flower[4 * l + 1] = lin(i, within(j + 1, 1));
      flower[4 * l + 2] = lin(within(i - 1, 0), j);
      flower[4 * l + 3] = lin(i, within(j - 1, 1));
    }
  }

  // model.hh:259-290
  double formation_per_supercell() const {
    if (use_nlist) {
      double e = 0.0;
      for (long l = 0; l < n(); ++l) e += occ[l] * (occ[nlist[2 * l]] + occ[nlist[2 * l + 1]]);
      e *= -J;
      return e;
    }
    double e = 0.0;
    for (long i = 0; i < rows; ++i) {
      long in = within(i + 1, 0);
      long dot = 0;
      for (long j = 0; j < cols; ++j) dot += (long)occ[lin(i, j)] * occ[lin(in, j)];
      e += -J * (double)dot;
    }
    for (long j = 0; j < cols; ++j) {
      long jn = within(j + 1, 1);
      long dot = 0;
      for (long i = 0; i < rows; ++i) dot += (long)occ[lin(i, j)] * occ[lin(i, jn)];
      e += -J * (double)dot;
    }
    return e;
  }

  // model.hh:305-345 (both branches compute the same expression tree)
  double delta_formation(long l, int new_occ) const {
    if (use_nlist) {
      return -J * (new_occ - occ[l]) *
             (occ[flower[4 * l]] + occ[flower[4 * l + 1]] + occ[flower[4 * l + 2]] + occ[flower[4 * l + 3]]);
    }
    long i = l % rows, j = l / rows;
    double ds = new_occ - occ[l];
    return -J * ds *
           (occ[lin(i, within(j - 1, 1))] + occ[lin(i, within(j + 1, 1))] +
            occ[lin(within(i - 1, 0), j)] + occ[lin(within(i + 1, 0), j)]);
  }

  // model.hh:410-416
  double Nx() const {
    long s = 0;
    for (long l = 0; l < n(); ++l) s += occ[l];
    return static_cast<double>(n() + s) / 2.0;
  }
};

struct IsingRunResult {
  SamplerMap samplers;
  long n_pass = 0;
  long long n_accept = 0, n_reject = 0;
  CompletionCheckResults results;
  long n_checks = 0;
};

// basic_semigrand_canonical.hh:416-470 + basic_occupation_metropolis.hh:354-425 with the
// default sampling functions (:486-590): "param_composition", "formation_energy",
// "potential_energy".  Clock time is supplied as 0 (no clock-time cutoffs in tests).
inline IsingRunResult run_ising_sgc(IsingModel& m, double temperature, double mu,
                                    const CompletionCheckParams& ccp, int sample_period,
                                    std::mt19937_64& engine) {
  if (m.use_nlist) m.build_nlist();
  IsingRunResult R;
  R.samplers.emplace("param_composition", Sampler(1));
  R.samplers.emplace("formation_energy", Sampler(1));
  R.samplers.emplace("potential_energy", Sampler(1));
  Sampler sample_weight(1);
  CompletionCheck cc(ccp);
  double beta = 1.0 / (KB * temperature);
  RNG rng{&engine};
  long max_l = m.n() - 1;
  long n_steps_per_pass = m.n();
  long n_pass_next_sample = sample_period;
  long n_step = 0;
  const double n_uc = (double)m.n();
  while (!cc.is_complete(R.samplers, sample_weight, R.n_pass, std::nullopt, 0.0)) {
    long l = rng.random_int(max_l);
    int new_occ = -m.occ[l];
    double dEf = m.delta_formation(l, new_occ);
    double Ndx = 0.0;
    Ndx += (new_occ - m.occ[l]) / 2.0;
    double dE = dEf - mu * Ndx;
    if (metropolis_acceptance(dE, beta, rng)) {
      R.n_accept++;
      m.occ[l] = new_occ;
    } else {
      R.n_reject++;
    }
    n_step++;
    if (n_step == n_steps_per_pass) {
      n_step = 0;
      R.n_pass += 1;
    }
    if (R.n_pass == n_pass_next_sample) {
      n_pass_next_sample += sample_period;
      // samplers are filled in map (name) order; each is a pure function of the state
      double Nx = m.Nx();
      double Ef = m.formation_per_supercell();
      R.samplers.at("formation_energy").push_back({Ef / n_uc});
      R.samplers.at("param_composition").push_back({Nx / n_uc});
      R.samplers.at("potential_energy").push_back({(Ef - mu * Nx) / n_uc});
    }
  }
  R.results = cc.results();
  R.n_checks = cc.n_checks();
  return R;
}

}  // namespace oracle

// ORACLE (test infrastructure only): C entry points over the CPU restatement, loaded
// with ctypes by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.  Never
// part of the product path.
#include <chrono>
#include <cstring>
#include <random>
#include <sstream>
#include <string>

#include "oracle_ce.hh"

using namespace oracle;

namespace {

std::string g_engine_state;

void load_engine(std::mt19937_64& e, const char* state) {
  std::stringstream ss(state);
  ss >> e;
}

}  // namespace

extern "C" {

struct OrcCCParams {
  int has_min_count, has_min_sample, has_max_count, has_max_sample;
  long min_count, min_sample, max_count, max_sample;
  int log_spacing;
  long check_begin, check_period;
  double check_base, check_shift;
  long check_period_max;
  double confidence;
  // requested precision for up to 4 sampler components (sampler index into the run's
  // sampler names, component index)
  int n_req;
  int req_sampler[4];
  int req_component[4];
  int req_abs_flag[4];
  double req_abs[4];
  int req_rel_flag[4];
  double req_rel[4];
};

struct OrcRunOut {
  long n_pass;
  long long n_accept, n_reject;
  long n_samples;
  int is_complete, all_equilibrated, all_converged;
  long n_checks;
  long N_samples_for_all_to_equilibrate;
  long N_samples_for_statistics;
  double mean[4];
  double calculated_precision[4];
  int is_converged[4];
};

// the 10000th output of a default-constructed std::mt19937_64 ([rand.predef])
unsigned long long orc_mt19937_64_10000th() {
  std::mt19937_64 e;
  e.discard(9999);
  return e();
}

// Draws from the reference's RandomNumberGenerator: kind 0 = random_int(max_i),
// kind 1 = random_real(max_r); engine state in/out as text (operator<< format).
int orc_rng_draws(const char* state_in, int kind, long max_i, double max_r, long n, long* out_i,
                  double* out_r, char* state_out, long state_len) {
  std::mt19937_64 e;
  load_engine(e, state_in);
  RNG rng{&e};
  for (long i = 0; i < n; ++i) {
    if (kind == 0)
      out_i[i] = rng.random_int(max_i);
    else
      out_r[i] = rng.random_real(max_r);
  }
  std::stringstream ss;
  ss << e;
  std::string s = ss.str();
  if ((long)s.size() + 1 > state_len) return -1;
  std::memcpy(state_out, s.c_str(), s.size() + 1);
  return 0;
}

// Semi-grand canonical proposals with the reference's occupant tracking, for a supercell
// whose n_sites sites all allow the same n_species occupants (one asymmetric unit):
// candidates (asym 0, species s) in species order; swaps a -> b for every ordered pair
// a != b (OccCandidate.cc:125-140); each step draws the swap type with
// random_real(sum of cand_size(a)) against the running sums and the site with
// random_int(cand_size(a) - 1) (OccEventProposal.hh:168-247), then (if apply) applies the
// event by swap-remove (OccLocation.cc:212-245).  Writes the proposed (site, new occupant).
int orc_sgc_proposals(long n_sites, int n_species, const int* occ_in, unsigned long long seed, long n_steps,
                      int apply, long* l_out, int* new_occ_out) {
  std::mt19937_64 e(seed);
  RNG rng{&e};
  std::vector<std::vector<long>> loc(n_species);
  std::vector<long> mol_loc(n_sites);
  std::vector<int> species(occ_in, occ_in + n_sites);
  for (long l = 0; l < n_sites; ++l) {
    if (species[l] < 0 || species[l] >= n_species) return -1;
    mol_loc[l] = (long)loc[species[l]].size();
    loc[species[l]].push_back(l);
  }
  std::vector<std::pair<int, int>> swaps;
  for (int a = 0; a < n_species; ++a)
    for (int b = 0; b < n_species; ++b)
      if (a != b) swaps.push_back({a, b});
  std::vector<double> tsum(swaps.size() + 1);
  for (long t = 0; t < n_steps; ++t) {
    tsum[0] = 0.0;
    for (size_t i = 0; i < swaps.size(); ++i) tsum[i + 1] = tsum[i] + (double)loc[swaps[i].first].size();
    if (tsum.back() == 0.0) return -2;
    const double r = rng.random_real(tsum.back());
    size_t k = 0;
    while (k < swaps.size() && !(r < tsum[k + 1])) ++k;
    if (k == swaps.size()) return -3;
    const int a = swaps[k].first, b = swaps[k].second;
    const long l = loc[a][rng.random_int((long)loc[a].size() - 1)];
    l_out[t] = l;
    new_occ_out[t] = b;
    if (apply) {
      const long back = loc[a].back();
      loc[a][mol_loc[l]] = back;
      mol_loc[back] = mol_loc[l];
      loc[a].pop_back();
      mol_loc[l] = (long)loc[b].size();
      loc[b].push_back(l);
      species[l] = b;
    }
  }
  return 0;
}

int orc_engine_seed(unsigned long long seed, char* state_out, long state_len) {
  std::mt19937_64 e(seed);
  std::stringstream ss;
  ss << e;
  std::string s = ss.str();
  if ((long)s.size() + 1 > state_len) return -1;
  std::memcpy(state_out, s.c_str(), s.size() + 1);
  return 0;
}

// Ising semi-grand canonical run with the reference's semantics.  samplers are
// "formation_energy"(0), "param_composition"(1), "potential_energy"(2) (map order).
int orc_ising_run(long rows, long cols, double J, int use_nlist, double T, double mu, int* occ,
                  const OrcCCParams* p, int sample_period, const char* engine_state,
                  double* samples_out, long max_samples, OrcRunOut* out, char* state_out,
                  long state_len) {
  try {
    IsingModel m;
    m.rows = rows;
    m.cols = cols;
    m.J = J;
    m.use_nlist = use_nlist != 0;
    m.occ.assign(occ, occ + rows * cols);
    CompletionCheckParams ccp;
    if (p->has_min_count) ccp.cutoff_params.min_count = p->min_count;
    if (p->has_min_sample) ccp.cutoff_params.min_sample = p->min_sample;
    if (p->has_max_count) ccp.cutoff_params.max_count = p->max_count;
    if (p->has_max_sample) ccp.cutoff_params.max_sample = p->max_sample;
    ccp.log_spacing = p->log_spacing != 0;
    ccp.check_begin = p->check_begin;
    ccp.check_period = p->check_period;
    ccp.check_base = p->check_base;
    ccp.check_shift = p->check_shift;
    ccp.check_period_max = p->check_period_max;
    ccp.calc_statistics.confidence = p->confidence;
    const char* names[3] = {"formation_energy", "param_composition", "potential_energy"};
    std::vector<SamplerComponent> keys;
    for (int r = 0; r < p->n_req; ++r) {
      SamplerComponent k{names[p->req_sampler[r]], p->req_component[r]};
      RequestedPrecision rp;
      rp.abs_convergence_is_required = p->req_abs_flag[r] != 0;
      rp.abs_precision = p->req_abs[r];
      rp.rel_convergence_is_required = p->req_rel_flag[r] != 0;
      rp.rel_precision = p->req_rel[r];
      ccp.requested_precision[k] = rp;
      keys.push_back(k);
    }
    std::mt19937_64 e;
    load_engine(e, engine_state);
    IsingRunResult R = run_ising_sgc(m, T, mu, ccp, sample_period, e);
    std::memcpy(occ, m.occ.data(), sizeof(int) * m.occ.size());
    long ns = get_n_samples(R.samplers);
    out->n_samples = ns;
    for (int s = 0; s < 3; ++s) {
      const auto& col = R.samplers.at(names[s]).cols[0];
      for (long i = 0; i < ns && i < max_samples; ++i) samples_out[s * max_samples + i] = col[i];
    }
    out->n_pass = R.n_pass;
    out->n_accept = R.n_accept;
    out->n_reject = R.n_reject;
    out->is_complete = R.results.is_complete;
    out->all_equilibrated = R.results.equilibration_check_results.all_equilibrated;
    out->all_converged = R.results.convergence_check_results.all_converged;
    out->n_checks = R.n_checks;
    out->N_samples_for_all_to_equilibrate =
        R.results.equilibration_check_results.N_samples_for_all_to_equilibrate;
    out->N_samples_for_statistics = R.results.convergence_check_results.N_samples_for_statistics;
    for (size_t r = 0; r < keys.size(); ++r) {
      auto& ir = R.results.convergence_check_results.individual_results;
      auto it = ir.find(keys[r]);
      if (it != ir.end()) {
        out->mean[r] = it->second.stats.mean;
        out->calculated_precision[r] = it->second.stats.calculated_precision;
        out->is_converged[r] = it->second.is_converged;
      } else {
        out->mean[r] = 0.0;
        out->calculated_precision[r] = -1.0;
        out->is_converged[r] = 0;
      }
    }
    std::stringstream ss;
    ss << e;
    std::string s = ss.str();
    if ((long)s.size() + 1 > state_len) return -1;
    std::memcpy(state_out, s.c_str(), s.size() + 1);
    return 0;
  } catch (std::exception&) {
    return -2;
  }
}

// Ising ΔE / energies for known-answer checks
double orc_ising_delta(long rows, long cols, double J, int use_nlist, const int* occ, long l,
                       int new_occ, double mu) {
  IsingModel m{rows, cols, J, use_nlist != 0, std::vector<int>(occ, occ + rows * cols), {}, {}};
  if (m.use_nlist) m.build_nlist();
  double dEf = m.delta_formation(l, new_occ);
  double Ndx = 0.0;
  Ndx += (new_occ - m.occ[l]) / 2.0;
  return dEf - mu * Ndx;
}
double orc_ising_formation(long rows, long cols, double J, int use_nlist, const int* occ) {
  IsingModel m{rows, cols, J, use_nlist != 0, std::vector<int>(occ, occ + rows * cols), {}, {}};
  if (m.use_nlist) m.build_nlist();
  return m.formation_per_supercell();
}

// statistics
void orc_equilibration_check(const double* obs, long n, double prec, int* is_eq, long* n_eq) {
  auto r = default_equilibration_check_raw(obs, n, prec);
  *is_eq = r.is_equilibrated;
  *n_eq = r.N_samples_for_equilibration;
}
void orc_basic_statistics(const double* obs, long n, const double* w, long nw, double confidence,
                          long method, long n_resamples, double* mean, double* prec) {
  BasicStatisticsCalculator c;
  c.confidence = confidence;
  c.method = method;
  c.n_resamples = n_resamples;
  auto s = c(obs, n, w, nw);
  *mean = s.mean;
  *prec = s.calculated_precision;
}
double orc_autocorrelation_factor(const double* obs, long n, double increment) {
  return autocorrelation_factor(obs, n, increment);
}
double orc_approx_erf_inv(double x) { return approx_erf_inv(x); }

void orc_philox4x32_10(const unsigned int* ctr, const unsigned int* key, unsigned int* out) {
  auto r = philox4x32_10({ctr[0], ctr[1], ctr[2], ctr[3]}, {key[0], key[1]});
  for (int i = 0; i < 4; ++i) out[i] = r[i];
}

// ---- cluster expansion ----
void* orc_ce_create(long L0, long L1, long L2, int n_species, const double* V, int n_classes) {
  try {
    auto* S = new CESupercell();
    S->L0 = L0;
    S->L1 = L1;
    S->L2 = L2;
    S->basis = make_oracle_basis(n_species);
    S->build();
    if ((int)S->classes.size() != n_classes) {
      delete S;
      return nullptr;
    }
    S->V.assign(V, V + n_classes);
    return S;
  } catch (std::exception&) {
    return nullptr;
  }
}
void orc_ce_destroy(void* h) { delete static_cast<CESupercell*>(h); }
int orc_ce_n_classes_for(int n_species) {
  return (int)enumerate_classes(make_oracle_basis(n_species)).size();
}
// class info: size, multiplicity, decoration multiset packed as base-4 digits
void orc_ce_class_info(int n_species, int* sizes, long* mults, long* decor_code) {
  auto cls = enumerate_classes(make_oracle_basis(n_species));
  for (size_t c = 0; c < cls.size(); ++c) {
    sizes[c] = cls[c].size;
    mults[c] = cls[c].multiplicity;
    long code = 0;
    for (int b : cls[c].decoration) code = code * 4 + (b + 1);
    decor_code[c] = code;
  }
}
double orc_ce_delta_e(void* h, const int* occ, long l, int new_occ, const double* mu, int n_mu) {
  auto* S = static_cast<CESupercell*>(h);
  std::vector<double> m(mu, mu + n_mu);
  return S->delta_formation(occ, l, new_occ) - S->mu_dot_Ndx(m, occ[l], new_occ);
}
double orc_ce_formation(void* h, const int* occ) {
  return static_cast<CESupercell*>(h)->formation_per_supercell(occ);
}
void orc_ce_int_corr(void* h, const int* occ, long long* out) {
  auto C = static_cast<CESupercell*>(h)->int_corr(occ);
  for (size_t i = 0; i < C.size(); ++i) out[i] = C[i];
}
int orc_ce_colored_sweep(void* h, int* occ, double T, const double* mu, int n_mu,
                         unsigned long long seed, unsigned int chain, const int* color,
                         int n_colors, long pass0, long n_passes, long long* corr_out,
                         long long* nacc_out) {
  auto* S = static_cast<CESupercell*>(h);
  std::vector<double> m(mu, mu + n_mu);
  std::vector<int> col(color, color + S->n());
  auto R = colored_sweep(*S, occ, T, m, seed, chain, col, n_colors, pass0, n_passes);
  long nc = (long)S->classes.size();
  for (long p = 0; p < n_passes; ++p) {
    for (long c = 0; c < nc; ++c) corr_out[p * nc + c] = R.corr[p][c];
    nacc_out[p] = R.n_accept[p];
  }
  return 0;
}

// The reference's random-site semi-grand canonical loop (basic_semigrand_canonical.hh:
// 308-320 proposal, basic_occupation_metropolis.hh:381-404 accept/apply) with the
// clexulator-style CE potential; used as the timed CPU baseline.  Binary: o -> 1-o;
// ternary: the other two species with equal probability (the SGC swap distribution of
// OccEventProposal.hh:260-336).  Returns accepted steps; *seconds = wall time.
long long orc_ce_random_site_run(void* h, int* occ, double T, const double* mu, int n_mu,
                                 unsigned long long seed, long long n_steps, double* seconds) {
  auto* S = static_cast<CESupercell*>(h);
  std::vector<double> m(mu, mu + n_mu);
  std::mt19937_64 e(seed);
  RNG rng{&e};
  double beta = 1.0 / (KB * T);
  long max_l = S->n() - 1;
  long long nacc = 0;
  auto t0 = std::chrono::steady_clock::now();
  for (long long s = 0; s < n_steps; ++s) {
    long l = rng.random_int(max_l);
    int o = occ[l];
    int o2 = (S->basis.n_species == 2) ? 1 - o : (o + 1 + (int)rng.random_int(1L)) % 3;
    double dE = S->delta_formation(occ, l, o2) - S->mu_dot_Ndx(m, o, o2);
    if (metropolis_acceptance(dE, beta, rng)) {
      occ[l] = o2;
      ++nacc;
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  *seconds = std::chrono::duration<double>(t1 - t0).count();
  return nacc;
}

// Semi-grand canonical run of the cluster expansion with the reference's proposal and
// acceptance (one asymmetric unit, all species allowed): swap type a -> b drawn with
// random_real against running sums of cand_size(a), site with random_int(cand_size(a)-1)
// (OccEventProposal.hh:168-247), metropolis_acceptance (metropolis.hh:26-35), occupant
// lists updated by swap-remove (OccLocation.cc:212-245).  After every pass of N steps:
// e_out[p] = potential energy per site (E_f - sum_i mu_i N_(i+1)) / N, x_out[p][i] =
// N_(i+1) / N (E_f tracked by adding the FP64 change of every accepted proposal).  Returns
// the accepted count, or -1 on bad input.
long long orc_ce_sgc_samples(void* h, int* occ, double T, const double* mu, int n_mu, unsigned long long seed,
                             long n_passes, double* e_out, double* x_out) {
  auto* S = static_cast<CESupercell*>(h);
  const int ns = S->basis.n_species;
  if (n_mu != ns - 1) return -1;
  std::vector<double> m(mu, mu + n_mu);
  std::mt19937_64 e(seed);
  RNG rng{&e};
  const double beta = 1.0 / (KB * T);
  const long N = S->n();
  std::vector<std::vector<long>> loc(ns);
  std::vector<long> mol_loc(N);
  for (long l = 0; l < N; ++l) {
    if (occ[l] < 0 || occ[l] >= ns) return -1;
    mol_loc[l] = (long)loc[occ[l]].size();
    loc[occ[l]].push_back(l);
  }
  std::vector<std::pair<int, int>> swaps;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b)
      if (a != b) swaps.push_back({a, b});
  std::vector<double> tsum(swaps.size() + 1);
  long long nacc = 0;
  double Ef = S->formation_per_supercell(occ);  // tracked by accepted changes
  for (long p = 0; p < n_passes; ++p) {
    for (long t = 0; t < N; ++t) {
      tsum[0] = 0.0;
      for (size_t i = 0; i < swaps.size(); ++i) tsum[i + 1] = tsum[i] + (double)loc[swaps[i].first].size();
      const double r = rng.random_real(tsum.back());
      size_t k = 0;
      while (k + 1 < swaps.size() && !(r < tsum[k + 1])) ++k;
      const int a = swaps[k].first, b = swaps[k].second;
      const long l = loc[a][rng.random_int((long)loc[a].size() - 1)];
      const double dEf = S->delta_formation(occ, l, b);
      const double dE = dEf - S->mu_dot_Ndx(m, a, b);
      if (metropolis_acceptance(dE, beta, rng)) {
        ++nacc;
        Ef += dEf;
        const long back = loc[a].back();
        loc[a][mol_loc[l]] = back;
        mol_loc[back] = mol_loc[l];
        loc[a].pop_back();
        mol_loc[l] = (long)loc[b].size();
        loc[b].push_back(l);
        occ[l] = b;
      }
    }
    double Esgc = Ef;
    for (int i = 0; i < ns - 1; ++i) {
      const double Ni = (double)loc[i + 1].size();
      Esgc -= m[i] * Ni;
      x_out[p * (ns - 1) + i] = Ni / (double)N;
    }
    e_out[p] = Esgc / (double)N;
  }
  return nacc;
}

// The same semi-grand canonical dynamics as orc_ce_sgc_samples from a given engine state
// (std::mt19937_64 text form, as operator<< writes it), for the serial-replay comparison:
// per pass the accepted count nacc_out[p], the potential energy per site e_out[p] (E_f
// tracked by accepted FP64 changes) and x_out[p][i]; at the end the occupant lists
// (OccLocation::m_loc per species, list order) in loc_out with their sizes in
// loc_sizes_out[ns], and the engine state in state_out.  Returns the accepted count, or -1.
long long orc_ce_sgc_run(void* h, int* occ, double T, const double* mu, int n_mu, const char* engine_state,
                         long n_passes, double* e_out, double* x_out, long long* nacc_out, int* loc_sizes_out,
                         int* loc_out, char* state_out, long state_len) {
  auto* S = static_cast<CESupercell*>(h);
  const int ns = S->basis.n_species;
  if (n_mu != ns - 1) return -1;
  std::vector<double> m(mu, mu + n_mu);
  std::mt19937_64 e;
  {
    std::stringstream in(engine_state);
    in >> e;
    if (in.fail()) return -1;
  }
  RNG rng{&e};
  const double beta = 1.0 / (KB * T);
  const long N = S->n();
  std::vector<std::vector<long>> loc(ns);
  std::vector<long> mol_loc(N);
  for (long l = 0; l < N; ++l) {
    if (occ[l] < 0 || occ[l] >= ns) return -1;
    mol_loc[l] = (long)loc[occ[l]].size();
    loc[occ[l]].push_back(l);
  }
  std::vector<std::pair<int, int>> swaps;  // OccCandidate.cc:136-152 order for one asymmetric unit
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b)
      if (a != b) swaps.push_back({a, b});
  std::vector<double> tsum(swaps.size() + 1);
  long long nacc = 0;
  double Ef = S->formation_per_supercell(occ);
  for (long p = 0; p < n_passes; ++p) {
    long long pass_acc = 0;
    for (long t = 0; t < N; ++t) {
      tsum[0] = 0.0;
      for (size_t i = 0; i < swaps.size(); ++i) tsum[i + 1] = tsum[i] + (double)loc[swaps[i].first].size();
      if (tsum.back() == 0.0) return -1;
      const double r = rng.random_real(tsum.back());
      size_t k = swaps.size();
      for (size_t i = 0; i < swaps.size(); ++i)
        if (r < tsum[i + 1]) {
          k = i;
          break;
        }
      if (k == swaps.size()) return -1;  // the reference throws here
      const int a = swaps[k].first, b = swaps[k].second;
      const long l = loc[a][(size_t)std::uniform_int_distribution<unsigned long>(0, loc[a].size() - 1)(e)];
      const double dEf = S->delta_formation(occ, l, b);
      const double dE = dEf - S->mu_dot_Ndx(m, a, b);
      if (metropolis_acceptance(dE, beta, rng)) {
        ++nacc;
        ++pass_acc;
        Ef += dEf;
        const long back = loc[a].back();
        loc[a][mol_loc[l]] = back;
        mol_loc[back] = mol_loc[l];
        loc[a].pop_back();
        mol_loc[l] = (long)loc[b].size();
        loc[b].push_back(l);
        occ[l] = b;
      }
    }
    nacc_out[p] = pass_acc;
    double Esgc = Ef;
    for (int i = 0; i < ns - 1; ++i) {
      const double Ni = (double)loc[i + 1].size();
      Esgc -= m[i] * Ni;
      x_out[p * (ns - 1) + i] = Ni / (double)N;
    }
    e_out[p] = Esgc / (double)N;
  }
  long off = 0;
  for (int s = 0; s < ns; ++s) {
    loc_sizes_out[s] = (int)loc[s].size();
    for (long v : loc[s]) loc_out[off++] = (int)v;
  }
  std::stringstream ss;
  ss << e;
  const std::string st = ss.str();
  if ((long)st.size() + 1 > state_len) return -1;
  std::memcpy(state_out, st.c_str(), st.size() + 1);
  return nacc;
}

int orc_ce_canonical_sweep(void* h, int* occ, double T, unsigned long long seed, unsigned int chain,
                           const int* color_a, int n_a, const int* color_b, int n_b, const int* order_a,
                           const int* order_b, long pass0, long n_passes, long long* corr_out, long long* nacc_out) {
  auto* S = static_cast<CESupercell*>(h);
  std::vector<int> ca(color_a, color_a + S->n()), cb(color_b, color_b + S->n());
  std::vector<long> oa, ob;
  if (order_a) oa.assign(order_a, order_a + S->n());
  if (order_b) ob.assign(order_b, order_b + S->n());
  auto R = colored_canonical_sweep(*S, occ, T, seed, chain, ca, n_a, cb, n_b, pass0, n_passes, oa, ob);
  const long nc = (long)S->classes.size();
  for (long p = 0; p < n_passes; ++p) {
    for (long c = 0; c < nc; ++c) corr_out[p * nc + c] = R.corr[p][c];
    nacc_out[p] = R.n_accept[p];
  }
  return 0;
}

// The reference's canonical dynamics: N steps per pass, each the canonical event of
// OccEventProposal.hh:108-237 (swap type (a, b), a < b, chosen with weight n_a n_b by
// random_real; then an atom of each species by random_int over the occupant lists, as
// OccLocation::choose_mol) accepted by metropolis.hh:26-35 with the exact formation-energy
// change of the swap (the second site's change evaluated after the first is applied, so
// pairs sharing a cluster are exact).  Per pass: formation energy per site (tracked by
// accepted changes).  Returns the accepted count.
long long orc_ce_canonical_samples(void* h, int* occ, double T, unsigned long long seed, long n_passes,
                                   double* e_out) {
  auto* S = static_cast<CESupercell*>(h);
  const int ns = S->basis.n_species;
  std::mt19937_64 e(seed);
  RNG rng{&e};
  const double beta = 1.0 / (KB * T);
  const long N = S->n();
  std::vector<std::vector<long>> loc(ns);
  std::vector<long> mol_loc(N);
  for (long l = 0; l < N; ++l) {
    if (occ[l] < 0 || occ[l] >= ns) return -1;
    mol_loc[l] = (long)loc[occ[l]].size();
    loc[occ[l]].push_back(l);
  }
  std::vector<std::pair<int, int>> swaps;
  for (int a = 0; a < ns; ++a)
    for (int b = a + 1; b < ns; ++b) swaps.push_back({a, b});
  std::vector<double> tsum(swaps.size() + 1);
  long long nacc = 0;
  double Ef = S->formation_per_supercell(occ);
  for (long p = 0; p < n_passes; ++p) {
    for (long t = 0; t < N; ++t) {
      tsum[0] = 0.0;
      for (size_t i = 0; i < swaps.size(); ++i)
        tsum[i + 1] = tsum[i] + (double)loc[swaps[i].first].size() * (double)loc[swaps[i].second].size();
      if (tsum.back() == 0.0) break;
      const double r = rng.random_real(tsum.back());
      size_t k = 0;
      while (k + 1 < swaps.size() && !(r < tsum[k + 1])) ++k;
      const int a = swaps[k].first, b = swaps[k].second;
      const long la = loc[a][rng.random_int((long)loc[a].size() - 1)];
      const long lb = loc[b][rng.random_int((long)loc[b].size() - 1)];
      const double dEa = S->delta_formation(occ, la, b);
      occ[la] = b;
      const double dEb = S->delta_formation(occ, lb, a);
      occ[la] = a;
      const double dE = dEa + dEb;
      if (metropolis_acceptance(dE, beta, rng)) {
        ++nacc;
        Ef += dE;
        occ[la] = b;
        occ[lb] = a;
        loc[a][mol_loc[la]] = lb;
        loc[b][mol_loc[lb]] = la;
        std::swap(mol_loc[la], mol_loc[lb]);
      }
    }
    e_out[p] = Ef / (double)N;
  }
  return nacc;
}

// Rejection-free (N-fold way) semi-grand canonical dynamics on the CPU: the loop of
// methods/nfold.hh:48-149 with an event selector over single-site flips of Metropolis rate
// min(1, exp(-beta dE)) (FP64, delta_formation), chosen by a Fenwick tree of the rates;
// after a flip the rates of the sites sharing a cluster with it (and its own) are
// recomputed.  Used as the timed CPU baseline of the GPU selector.  Returns the events run;
// *seconds = wall time, *time_out = the simulated time.
long long orc_ce_nfold_run(void* h, int* occ, double T, const double* mu, int n_mu, unsigned long long seed,
                           long long n_events, double* seconds, double* time_out) {
  auto* S = static_cast<CESupercell*>(h);
  if (S->basis.n_species != 2 || n_mu != 1) return -1;
  std::vector<double> m(mu, mu + n_mu);
  const double beta = 1.0 / (KB * T);
  const long N = S->n();
  const long ns = (long)S->slots.size();
  std::mt19937_64 e(seed);
  RNG rng{&e};
  std::vector<double> rate(N), tree(N + 1, 0.0);
  auto set_rate = [&](long l, double r) {
    const double d = r - rate[l];
    rate[l] = r;
    for (long x = l + 1; x <= N; x += x & -x) tree[x] += d;
  };
  auto site_rate = [&](long l) {
    const double dE = S->delta_formation(occ, l, 1 - occ[l]) - S->mu_dot_Ndx(m, occ[l], 1 - occ[l]);
    return dE <= 0.0 ? 1.0 : std::exp(-beta * dE);
  };
  for (long l = 0; l < N; ++l) set_rate(l, site_rate(l));
  long top = 1;
  while (top * 2 <= N) top *= 2;
  const auto t0 = std::chrono::steady_clock::now();
  double time = 0.0;
  for (long long ev = 0; ev < n_events; ++ev) {
    double R = 0.0;
    for (long x = N; x > 0; x -= x & -x) R += tree[x];
    double target = rng.random_real(R);
    long pos = 0;
    for (long step = top; step > 0; step >>= 1)
      if (pos + step <= N && tree[pos + step] <= target) {
        pos += step;
        target -= tree[pos];
      }
    const long l = std::min(pos, N - 1);
    time += -std::log(1.0 - rng.random_real(1.0)) / R;
    occ[l] = 1 - occ[l];
    set_rate(l, site_rate(l));
    const int32_t* nb = S->nbr.data() + l * ns;
    for (long q = 0; q < ns; ++q) set_rate(nb[q], site_rate(nb[q]));
  }
  *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *time_out = time;
  return n_events;
}

}  // extern "C"

/* C++ facade over the montegpu C-ABI: RAII handles whose methods throw std::runtime_error
 * with the library's "Error in ..." message (the reference reports failures the same way,
 * include/casm/monte/definitions.hh:108-113, and pybind maps them to RuntimeError).
 * Header-only; link libmontegpu.so. */
#ifndef MONTEGPU_HPP
#define MONTEGPU_HPP

#include <array>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "montegpu.h"

namespace montegpu {

inline void check(int status) {
  if (status != MG_OK) throw std::runtime_error(mg_last_error());
}

/* A handle owning a library object, released by `Destroy`. */
template <class T, int (*Destroy)(T*)>
class Handle {
 public:
  Handle() = default;
  explicit Handle(T* p) : p_(p) {}
  Handle(const Handle&) = delete;
  Handle& operator=(const Handle&) = delete;
  Handle(Handle&& o) noexcept : p_(std::exchange(o.p_, nullptr)) {}
  Handle& operator=(Handle&& o) noexcept {
    if (this != &o) {
      reset();
      p_ = std::exchange(o.p_, nullptr);
    }
    return *this;
  }
  ~Handle() { reset(); }
  T* get() const { return p_; }
  void reset() {
    if (p_) Destroy(p_);
    p_ = nullptr;
  }

 private:
  T* p_ = nullptr;
};

/* std::mt19937_64 with the reference's RandomNumberGenerator semantics
 * (RandomNumberGenerator.hh:15-42): random_int(max) in [0, max], random_real(max) in
 * [0, max). */
class RandomNumberEngine {
 public:
  explicit RandomNumberEngine(bool seed_from_device = true) {
    mg_engine* e = nullptr;
    check(mg_engine_create(seed_from_device ? 1 : 0, &e));
    h_ = H(e);
  }
  void seed(uint64_t value) { check(mg_engine_seed(h_.get(), value)); }
  void seed_seq(const std::vector<uint64_t>& values) {
    check(mg_engine_seed_seq(h_.get(), values.data(), values.size()));
  }
  std::string dump() const {
    std::vector<char> buf(16384);
    check(mg_engine_dump(h_.get(), buf.data(), buf.size()));
    return std::string(buf.data());
  }
  void load(const std::string& state) { check(mg_engine_load(h_.get(), state.c_str())); }
  uint64_t random_int(uint64_t max) {
    uint64_t v = 0;
    check(mg_engine_random_int(h_.get(), max, &v));
    return v;
  }
  double random_real(double max) {
    double v = 0.0;
    check(mg_engine_random_real(h_.get(), max, &v));
    return v;
  }
  mg_engine* get() const { return h_.get(); }

 private:
  using H = Handle<mg_engine, mg_engine_destroy>;
  H h_;
};

/* Cluster-expansion model: basis kind 0 (FCC binary, occupation basis) or 1 (FCC
 * ternary, Chebyshev basis) and one ECI per class. */
class CeModel {
 public:
  CeModel(int basis_kind, const std::vector<double>& eci) {
    mg_ce_model* m = nullptr;
    check(mg_ce_model_create(basis_kind, eci.data(), (int)eci.size(), &m));
    h_ = H(m);
    check(mg_ce_model_info(m, &n_classes_, &n_features_, &n_species_));
  }
  int n_classes() const { return n_classes_; }
  int n_species() const { return n_species_; }
  const mg_ce_model* get() const { return h_.get(); }

 private:
  using H = Handle<mg_ce_model, mg_ce_model_destroy>;
  H h_;
  int n_classes_ = 0, n_features_ = 0, n_species_ = 0;
};

/* Chains of one supercell shape resident on the GPU (mg_ce_batch_*). */
class CeBatch {
 public:
  CeBatch(const CeModel& m, int L0, int L1, int L2, const std::vector<double>& temperature,
          const std::vector<double>& mu, const std::vector<uint64_t>& seeds, const std::vector<int8_t>& occ,
          bool fp32_decisions = false, int ctas_per_chain = 0)
      : n_chains_((int)temperature.size()), n_sites_((long long)L0 * L1 * L2), n_slots_(m.n_classes() + 2) {
    mg_ce_batch* b = nullptr;
    check(mg_ce_batch_create(m.get(), L0, L1, L2, n_chains_, temperature.data(), mu.data(), seeds.data(), nullptr,
                             occ.data(), fp32_decisions ? 1 : 0, ctas_per_chain, &b));
    h_ = H(b);
  }
  /* per-pass outputs [n_passes][n_chains][n_classes + 2] */
  std::vector<long long> run(int n_passes) {
    std::vector<long long> out((size_t)n_passes * n_chains_ * n_slots_);
    check(mg_ce_batch_run(h_.get(), n_passes, out.data()));
    return out;
  }
  std::vector<int8_t> occupation() {
    std::vector<int8_t> occ((size_t)n_sites_ * n_chains_);
    check(mg_ce_batch_get_occ(h_.get(), occ.data()));
    return occ;
  }
  int layout() const {
    int l = 0;
    check(mg_ce_batch_layout(h_.get(), &l));
    return l;
  }
  void set_layout(int layout) { check(mg_ce_batch_set_layout(h_.get(), layout)); }
  float last_kernel_ms() const {
    float ms = 0.f;
    check(mg_ce_batch_last_kernel_ms(h_.get(), &ms));
    return ms;
  }
  /* rotation over two cluster sizes: {CTAs of the fast clusters (0: no rotation), measured
   * time ratio per pass fast / slow}; allow or forbid it; kernels launched by the last run */
  std::pair<int, double> rotation() const {
    int s = 0;
    double r = 0.0;
    check(mg_ce_batch_rotation(h_.get(), &s, &r));
    return {s, r};
  }
  void set_rotation(bool allowed) { check(mg_ce_batch_set_rotation(h_.get(), allowed ? 1 : 0)); }
  int last_launches() const {
    int n = 0;
    check(mg_ce_batch_last_launches(h_.get(), &n));
    return n;
  }
  mg_ce_batch* get() const { return h_.get(); }

 private:
  using H = Handle<mg_ce_batch, mg_ce_batch_destroy>;
  H h_;
  int n_chains_;
  long long n_sites_;
  int n_slots_;
};

/* Chains of one supercell swept at fixed composition (mg_ce_canon_*): exchanges of matched
 * same-colour sites, the canonical event of the reference made parallel. */
class CeCanon {
 public:
  CeCanon(const CeModel& m, int L0, int L1, int L2, const std::vector<double>& temperature,
          const std::vector<uint64_t>& seeds, const std::vector<int8_t>& occ, bool fp32_decisions = false)
      : n_chains_((int)temperature.size()), n_sites_((long long)L0 * L1 * L2), n_slots_(m.n_classes() + 2) {
    mg_ce_canon* h = nullptr;
    check(mg_ce_canon_create(m.get(), L0, L1, L2, n_chains_, temperature.data(), seeds.data(), nullptr, occ.data(),
                             fp32_decisions ? 1 : 0, &h));
    h_ = H(h);
  }
  /* per-pass outputs [n_passes][n_chains][n_classes + 2], slot 0 accepted swaps */
  std::vector<long long> run(int n_passes) {
    std::vector<long long> out((size_t)n_passes * n_chains_ * n_slots_);
    check(mg_ce_canon_run(h_.get(), n_passes, out.data()));
    return out;
  }
  std::vector<int8_t> occupation() {
    std::vector<int8_t> occ((size_t)n_sites_ * n_chains_);
    check(mg_ce_canon_get_occ(h_.get(), occ.data()));
    return occ;
  }
  /* colouring `which` (0: even passes, 1: odd) and its list order */
  std::vector<int32_t> colors(int which) const {
    std::vector<int32_t> c((size_t)n_sites_);
    check(mg_ce_canon_colors(h_.get(), which, c.data()));
    return c;
  }
  std::vector<int32_t> class_order(int which) const {
    std::vector<int32_t> o((size_t)n_sites_);
    check(mg_ce_canon_class_order(h_.get(), which, o.data()));
    return o;
  }
  float last_kernel_ms() const {
    float ms = 0.f;
    check(mg_ce_canon_last_kernel_ms(h_.get(), &ms));
    return ms;
  }
  mg_ce_canon* get() const { return h_.get(); }

 private:
  using H = Handle<mg_ce_canon, mg_ce_canon_destroy>;
  H h_;
  int n_chains_;
  long long n_sites_;
  int n_slots_;
};

/* Rejection-free (N-fold way) dynamics of binary chains (mg_ce_nfold_*): per pass of N
 * events the pass's time, the total rate at its end and the time-weighted correlation sums. */
class CeNfold {
 public:
  CeNfold(const CeModel& m, int L0, int L1, int L2, const std::vector<double>& temperature,
          const std::vector<double>& mu, const std::vector<uint64_t>& seeds, const std::vector<int8_t>& occ)
      : n_chains_((int)temperature.size()), n_sites_((long long)L0 * L1 * L2), n_slots_(m.n_classes() + 2),
        n_classes_(m.n_classes()) {
    mg_ce_nfold* h = nullptr;
    check(mg_ce_nfold_create(m.get(), L0, L1, L2, n_chains_, temperature.data(), mu.data(), seeds.data(), nullptr,
                             occ.data(), &h));
    h_ = H(h);
  }
  /* [n_passes][n_chains][n_classes + 2] */
  std::vector<double> run(int n_passes) {
    std::vector<double> out((size_t)n_passes * n_chains_ * n_slots_);
    check(mg_ce_nfold_run(h_.get(), n_passes, out.data()));
    return out;
  }
  std::vector<int8_t> occupation() {
    std::vector<int8_t> occ((size_t)n_sites_ * n_chains_);
    check(mg_ce_nfold_get_occ(h_.get(), occ.data()));
    return occ;
  }
  /* integer correlation sums [n_chains][n_classes], tracked or recomputed */
  std::vector<long long> corr(bool recompute = false) {
    std::vector<long long> c((size_t)n_chains_ * n_classes_);
    check(mg_ce_nfold_corr(h_.get(), recompute ? 1 : 0, c.data()));
    return c;
  }
  float last_kernel_ms() const {
    float ms = 0.f;
    check(mg_ce_nfold_last_kernel_ms(h_.get(), &ms));
    return ms;
  }
  mg_ce_nfold* get() const { return h_.get(); }

 private:
  using H = Handle<mg_ce_nfold, mg_ce_nfold_destroy>;
  H h_;
  int n_chains_;
  long long n_sites_;
  int n_slots_, n_classes_;
};

/* Many chains of any supercell shapes in one HBM arena, swept by persistent kernels
 * (mg_ce_pool_*): the batched and served form of the per-chain run.  add / add_many throw
 * std::runtime_error on invalid input and return -1 / an empty vector when the arena or the
 * slots are full (MG_ERR_FULL: wait for running jobs and retry). */
class CePool {
 public:
  CePool(const CeModel& m, long long arena_bytes, int max_chains, bool fp32_decisions = false)
      : n_slots_(m.n_classes() + 2), n_classes_(m.n_classes()), n_species_(m.n_species()) {
    mg_ce_pool* p = nullptr;
    check(mg_ce_pool_create(m.get(), arena_bytes, max_chains, fp32_decisions ? 1 : 0, &p));
    h_ = H(p);
  }
  int add(int L0, int L1, int L2, double temperature, const std::vector<double>& mu, uint64_t seed,
          uint32_t chain_id, const std::vector<int8_t>& occ) {
    int slot = -1;
    const int rc = mg_ce_pool_add(h_.get(), L0, L1, L2, temperature, mu.data(), seed, chain_id, occ.data(), &slot);
    if (rc == MG_ERR_FULL) return -1;
    check(rc);
    shapes_[slot] = {L0, L1, L2};
    return slot;
  }
  /* n chains at once, all or none: dims [n][3], mu [n][n_species-1], occupations back to back */
  std::vector<int32_t> add_many(const std::vector<int32_t>& dims, const std::vector<double>& temperature,
                                const std::vector<double>& mu, const std::vector<uint64_t>& seeds,
                                const std::vector<uint32_t>& chain_ids, const std::vector<int8_t>& occ) {
    const int n = (int)temperature.size();
    if (dims.size() != 3 * (size_t)n || seeds.size() != (size_t)n || chain_ids.size() != (size_t)n ||
        mu.size() != (size_t)n * (n_species_ - 1))
      throw std::runtime_error("Error in CePool::add_many: argument sizes do not match");
    std::vector<int32_t> slots((size_t)n);
    const int rc = mg_ce_pool_add_many(h_.get(), n, dims.data(), temperature.data(), mu.data(), seeds.data(),
                                       chain_ids.data(), occ.data(), slots.data());
    if (rc == MG_ERR_FULL) return {};
    check(rc);
    for (int i = 0; i < n; ++i) shapes_[slots[i]] = {dims[3 * i], dims[3 * i + 1], dims[3 * i + 2]};
    return slots;
  }
  void remove(int slot) {
    check(mg_ce_pool_remove(h_.get(), slot));
    shapes_.erase(slot);
  }
  /* per-pass outputs [slot][n_passes][n_classes + 2] in the order of `slots` */
  std::vector<long long> run(const std::vector<int32_t>& slots, int n_passes) {
    std::vector<long long> out(slots.size() * (size_t)n_passes * n_slots_);
    check(mg_ce_pool_run(h_.get(), slots.data(), (int)slots.size(), n_passes, out.data()));
    return out;
  }
  std::vector<int8_t> occupation(int slot) {
    const auto it = shapes_.find(slot);
    if (it == shapes_.end()) throw std::runtime_error("Error in CePool::occupation: invalid slot");
    std::vector<int8_t> occ((size_t)it->second[0] * it->second[1] * it->second[2]);
    check(mg_ce_pool_get_occ(h_.get(), slot, occ.data()));
    return occ;
  }
  std::vector<long long> corr(int slot) {
    std::vector<long long> c((size_t)n_classes_);
    check(mg_ce_pool_corr(h_.get(), slot, c.data()));
    return c;
  }
  float last_kernel_ms() const {
    float ms = 0.f;
    check(mg_ce_pool_last_kernel_ms(h_.get(), &ms));
    return ms;
  }
  int last_launches() const {
    int n = 0;
    check(mg_ce_pool_last_launches(h_.get(), &n));
    return n;
  }
  mg_ce_pool* get() const { return h_.get(); }

 private:
  using H = Handle<mg_ce_pool, mg_ce_pool_destroy>;
  H h_;
  int n_slots_, n_classes_, n_species_;
  std::map<int, std::array<int, 3>> shapes_;
};

/* free the device blocks and streams that destroyed batches left in the library's cache */
inline void release_cached_memory() { check(mg_release_cached_memory()); }

/* The sweep's colouring of a supercell (host only): colours per site, number of
 * colours, layout (0 byte, 1 word, 2 pipelined word). */
struct Colouring {
  std::vector<int32_t> color;
  int n_colors = 0;
  int layout = 0;
};
inline Colouring color_supercell(int basis_kind, int L0, int L1, int L2) {
  Colouring c;
  c.color.resize((size_t)L0 * L1 * L2);
  const int n = mg_ce_color_supercell(basis_kind, L0, L1, L2, c.color.data(), &c.layout);
  if (n <= 0) throw std::runtime_error(mg_last_error());
  c.n_colors = n;
  return c;
}

/* BasicStatisticsCalculator (BasicStatistics.cc:114-188), unweighted: mean and the
 * autocorrelation-corrected precision of the mean. */
inline std::pair<double, double> basic_statistics(const std::vector<double>& obs, double confidence = 0.95) {
  double mean = 0.0, precision = 0.0;
  check(mg_basic_statistics(obs.data(), (long)obs.size(), nullptr, 0, confidence, 1, 10000, &mean, &precision));
  return {mean, precision};
}

/* _default_equilibration_check (EquilibrationCheck.cc:50-117): (equilibrated, samples
 * needed to equilibrate). */
inline std::pair<bool, long> equilibration_check(const std::vector<double>& obs, double precision) {
  int eq = 0;
  long n = 0;
  check(mg_equilibration_check(obs.data(), (long)obs.size(), precision, &eq, &n));
  return {eq != 0, n};
}

}  // namespace montegpu

#endif /* MONTEGPU_HPP */

// ORACLE (test infrastructure only): FCC cluster-expansion energy and semi-grand
// canonical Metropolis, restated on the CPU in FP64.
//
// The reference toolkit has no in-tree cluster-expansion evaluator (the evaluator lives
// in the external libcasm-clexulator, which is not a dependency of the package; parity
// of the CE numbers is therefore unpinned by the reference).  This file restates the
// clexulator pattern of tests/unit/monte/data/OccClexulatorZrOTest/.../ZrO_Clexulator.cc
// :4478-4501 (delta point correlations: (phi(new)-phi(old)) x sum over clusters of the
// product of the other sites' site functions) with real-valued site functions, and plugs
// it into the semi-grand canonical potential of
// include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:165-192 (dE = dE_f - mu.N dx).
//
// The cluster set is enumerated here independently of the product (which generates its
// GPU code from a Python enumeration): FCC point group (48 signed permutations),
// pairs 1-4NN, the three smallest triplets and the NN tetrahedron, decorated-cluster
// orbits for multi-function bases, in the documented order (size, ascending squared pair
// distances, canonical form).
//
// Also here: a restatement of the coloured-sweep algorithm of the GPU kernels (Philox4x32-10
// keyed by (seed), counters as in sweep_counter below; one visit per site per pass in
// colour order), used to check those kernels trajectory-for-trajectory.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <functional>
#include <map>
#include <set>
#include <stdexcept>
#include <vector>

#include "oracle_ising.hh"

namespace oracle {

typedef std::array<long, 3> V3;
typedef std::array<long, 4> V4;  // x, y, z, basis index

inline std::vector<std::array<std::array<long, 3>, 3>> cubic_point_group() {
  std::vector<std::array<std::array<long, 3>, 3>> ops;
  int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  for (auto& p : perms)
    for (int s = 0; s < 8; ++s) {
      std::array<std::array<long, 3>, 3> m{};
      for (int r = 0; r < 3; ++r) m[r][p[r]] = (s >> r & 1) ? -1 : 1;
      ops.push_back(m);
    }
  return ops;
}

inline long d2(const V3& a, const V3& b) {
  long s = 0;
  for (int i = 0; i < 3; ++i) s += (a[i] - b[i]) * (a[i] - b[i]);
  return s;
}

// canonical form of a decorated cluster (decor may be all zero for plain clusters)
inline std::vector<V4> canon(const std::vector<V3>& sites, const std::vector<int>& decor) {
  static const auto ops = cubic_point_group();
  std::vector<V4> best;
  for (auto& g : ops) {
    std::vector<V4> t;
    for (size_t i = 0; i < sites.size(); ++i) {
      V4 v;
      for (int r = 0; r < 3; ++r) v[r] = g[r][0] * sites[i][0] + g[r][1] * sites[i][1] + g[r][2] * sites[i][2];
      v[3] = decor[i];
      t.push_back(v);
    }
    std::sort(t.begin(), t.end());
    V4 o = t[0];
    for (auto& v : t)
      for (int r = 0; r < 3; ++r) v[r] -= o[r];
    if (best.empty() || t < best) best = t;
  }
  return best;
}

inline std::vector<long> sorted_d2(const std::vector<V3>& s) {
  std::vector<long> out;
  for (size_t i = 0; i < s.size(); ++i)
    for (size_t j = i + 1; j < s.size(); ++j) out.push_back(d2(s[i], s[j]));
  std::sort(out.begin(), out.end());
  return out;
}

struct OracleClass {
  int size = 0;
  long multiplicity = 1;  // decorated clusters per primitive cell
  std::vector<int> decoration;  // sorted multiset of basis indices
  // members containing the origin: sites (Cartesian) and decoration
  std::vector<std::pair<std::vector<V3>, std::vector<int>>> members;
};

struct OracleBasis {
  int n_species = 2;
  std::vector<std::vector<int>> psi;  // psi[b][o]
  std::vector<double> scale;          // a[b]
  double phi(int b, int o) const { return scale[b] * psi[b][o]; }
};

inline OracleBasis make_oracle_basis(int n_species) {
  OracleBasis B;
  B.n_species = n_species;
  if (n_species == 2) {
    B.psi = {{0, 1}};
    B.scale = {1.0};
  } else if (n_species == 3) {
    B.psi = {{-1, 0, 1}, {1, -2, 1}};
    B.scale = {std::sqrt(1.5), 1.0 / std::sqrt(2.0)};
  } else {
    throw std::runtime_error("oracle: unsupported number of species");
  }
  return B;
}

inline bool is_fcc_site(const V3& v) {
  auto ev = [](long x) { return ((x % 2) + 2) % 2 == 0; };
  if (!ev(v[0]) || !ev(v[1]) || !ev(v[2])) return false;
  long h = (v[0] + v[1] + v[2]) / 2;
  return ((h % 2) + 2) % 2 == 0;
}

// Enumerate classes (empty, point, 4 pair shells, 3 triplets, 1 quad) for a basis.
inline std::vector<OracleClass> enumerate_classes(const OracleBasis& B) {
  const long d2max = 32;
  std::vector<V3> nbrs;
  for (long x = -6; x <= 6; ++x)
    for (long y = -6; y <= 6; ++y)
      for (long z = -6; z <= 6; ++z) {
        V3 v{x, y, z};
        if ((x || y || z) && is_fcc_site(v) && x * x + y * y + z * z <= d2max) nbrs.push_back(v);
      }
  std::sort(nbrs.begin(), nbrs.end());
  V3 O{0, 0, 0};
  // orbits as lists of clusters containing the origin
  std::vector<std::vector<std::vector<V3>>> orbits;
  orbits.push_back({{}});
  orbits.push_back({{O}});
  for (long s2 : {8L, 16L, 24L, 32L}) {
    std::vector<std::vector<V3>> cl;
    for (auto& v : nbrs)
      if (v[0] * v[0] + v[1] * v[1] + v[2] * v[2] == s2) cl.push_back({O, v});
    orbits.push_back(cl);
  }
  auto multi = [&](int k, int keep) {
    std::map<std::vector<V4>, std::vector<std::vector<V3>>> groups;
    std::vector<int> idx(k - 1);
    // combinations of nbrs of size k-1
    std::vector<int> sel;
    std::function<void(int, int)> rec = [&](int start, int depth) {
      if (depth == k - 1) {
        std::vector<V3> s{O};
        for (int i : sel) s.push_back(nbrs[i]);
        for (size_t a = 0; a < s.size(); ++a)
          for (size_t b = a + 1; b < s.size(); ++b)
            if (d2(s[a], s[b]) > d2max) return;
        groups[canon(s, std::vector<int>(s.size(), 0))].push_back(s);
        return;
      }
      for (int i = start; i < (int)nbrs.size(); ++i) {
        sel.push_back(i);
        rec(i + 1, depth + 1);
        sel.pop_back();
      }
    };
    rec(0, 0);
    std::vector<std::pair<std::pair<std::vector<long>, std::vector<V4>>, std::vector<std::vector<V3>>>> keyed;
    for (auto& kv : groups) keyed.push_back({{sorted_d2(kv.second[0]), kv.first}, kv.second});
    std::sort(keyed.begin(), keyed.end(),
              [](auto& a, auto& b) { return a.first < b.first; });
    for (int i = 0; i < keep && i < (int)keyed.size(); ++i) orbits.push_back(keyed[i].second);
  };
  multi(3, 3);
  multi(4, 1);

  int nb = (int)B.psi.size();
  std::vector<OracleClass> classes;
  for (auto& orb : orbits) {
    int size = (int)orb[0].size();
    if (size == 0) {
      OracleClass c;
      c.size = 0;
      c.multiplicity = 1;
      c.members.push_back({{}, {}});
      classes.push_back(c);
      continue;
    }
    std::map<std::vector<V4>, OracleClass> groups;
    long ndec = 1;
    for (int i = 0; i < size; ++i) ndec *= nb;
    for (auto& s : orb) {
      for (long code = 0; code < ndec; ++code) {
        std::vector<int> dec(size);
        long c = code;
        for (int i = size - 1; i >= 0; --i) {
          dec[i] = (int)(c % nb);
          c /= nb;
        }
        auto key = canon(s, dec);
        auto& g = groups[key];
        g.size = size;
        g.members.push_back({s, dec});
      }
    }
    for (auto& kv : groups) {
      OracleClass c = kv.second;
      c.multiplicity = (long)c.members.size() / size;
      c.decoration = c.members[0].second;
      std::sort(c.decoration.begin(), c.decoration.end());
      classes.push_back(c);
    }
  }
  return classes;
}

// primitive coordinates of a Cartesian FCC vector (lattice columns (0,2,2),(2,0,2),(2,2,0))
inline V3 cart_to_prim(const V3& v) {
  // inverse of [[0,2,2],[2,0,2],[2,2,0]] is 1/4 * [[-1,1,1],[1,-1,1],[1,1,-1]]
  long n0 = (-v[0] + v[1] + v[2]), n1 = (v[0] - v[1] + v[2]), n2 = (v[0] + v[1] - v[2]);
  if (n0 % 4 || n1 % 4 || n2 % 4) throw std::runtime_error("oracle: not a lattice vector");
  return V3{n0 / 4, n1 / 4, n2 / 4};
}

// A supercell L0 x L1 x L2 of the primitive cell; l = i + L0*(j + L1*k).
// Like a clexulator, cluster members are stored once as templates over neighbour
// slots (translation invariance) and a per-site neighbour table resolves the slots.
struct CESupercell {
  long L0, L1, L2;
  OracleBasis basis;
  std::vector<OracleClass> classes;
  std::vector<double> V;  // ECI per class (same order as classes)
  struct Member {
    int cls;
    int b_l;
    std::vector<std::pair<int, int>> others;  // (neighbour slot, basis index)
  };
  std::vector<V3> slots;                // prim offsets of the neighbour slots
  std::vector<Member> tmpl;             // members containing the changing site
  std::vector<int32_t> nbr;             // [site * slots.size() + slot]
  std::vector<std::vector<std::vector<std::pair<V3, int>>>> anchored;  // [class][i] -> (offset, b)

  long n() const { return L0 * L1 * L2; }
  static long wrap(long x, long L) { return ((x % L) + L) % L; }
  long index(long i, long j, long k) const { return wrap(i, L0) + L0 * (wrap(j, L1) + L1 * wrap(k, L2)); }

  void build() {
    classes = enumerate_classes(basis);
    std::map<V3, int> slot_of;
    tmpl.clear();
    for (size_t c = 0; c < classes.size(); ++c) {
      if (classes[c].size == 0) continue;
      for (auto& m : classes[c].members) {
        Member M;
        M.cls = (int)c;
        M.b_l = -1;
        for (size_t s = 0; s < m.first.size(); ++s) {
          const V3& v = m.first[s];
          if (v[0] == 0 && v[1] == 0 && v[2] == 0) {
            M.b_l = m.second[s];
            continue;
          }
          V3 p = cart_to_prim(v);
          auto it = slot_of.find(p);
          int slot;
          if (it == slot_of.end()) {
            slot = (int)slots.size();
            slots.push_back(p);
            slot_of[p] = slot;
          } else {
            slot = it->second;
          }
          M.others.push_back({slot, m.second[s]});
        }
        tmpl.push_back(M);
      }
    }
    long ns = (long)slots.size();
    nbr.assign(n() * ns, 0);
    for (long l = 0; l < n(); ++l) {
      long i = l % L0, j = (l / L0) % L1, k = l / (L0 * L1);
      for (long s = 0; s < ns; ++s)
        nbr[l * ns + s] = (int32_t)index(i + slots[s][0], j + slots[s][1], k + slots[s][2]);
    }
    anchored.assign(classes.size(), {});
    for (size_t c = 0; c < classes.size(); ++c) {
      if (classes[c].size == 0) continue;
      for (auto& m : classes[c].members) {
        V3 mn = *std::min_element(m.first.begin(), m.first.end());
        if (!(mn[0] == 0 && mn[1] == 0 && mn[2] == 0)) continue;
        std::vector<std::pair<V3, int>> t;
        for (size_t s = 0; s < m.first.size(); ++s) t.push_back({cart_to_prim(m.first[s]), m.second[s]});
        anchored[c].push_back(t);
      }
      if ((long)anchored[c].size() != classes[c].multiplicity)
        throw std::runtime_error("oracle: anchored count != multiplicity");
    }
  }

  // clexulator-style FP64 change of formation energy per supercell (real phi)
  mutable std::vector<double> acc_scratch;  // per-class sums of delta_formation

  double delta_formation(const int* occ, long l, int new_occ) const {
    int o = occ[l];
    std::vector<double>& acc = acc_scratch;
    acc.assign(classes.size(), 0.0);
    const int32_t* nb = nbr.data() + l * (long)slots.size();
    for (auto& M : tmpl) {
      double prod = basis.phi(M.b_l, new_occ) - basis.phi(M.b_l, o);
      for (auto& e : M.others) prod *= basis.phi(e.second, occ[nb[e.first]]);
      acc[M.cls] += prod;
    }
    double dE = 0.0;
    for (size_t c = 0; c < classes.size(); ++c) {
      if (classes[c].size == 0) continue;
      dE += V[c] * (acc[c] / (double)classes[c].multiplicity);
    }
    return dE;
  }

  // integer correlation sums: sum over each decorated cluster of prod psi
  std::vector<long long> int_corr(const int* occ) const {
    std::vector<long long> C(classes.size(), 0);
    for (long l = 0; l < n(); ++l) {
      long i = l % L0, j = (l / L0) % L1, k = l / (L0 * L1);
      C[0] += 1;
      for (size_t c = 1; c < classes.size(); ++c)
        for (auto& t : anchored[c]) {
          long long p = 1;
          for (auto& e : t) p *= basis.psi[e.second][occ[index(i + e.first[0], j + e.first[1], k + e.first[2])]];
          C[c] += p;
        }
    }
    return C;
  }

  // FP64 formation energy per supercell from correlations (CASM normalisation)
  double formation_per_supercell(const int* occ) const {
    auto C = int_corr(occ);
    double E = 0.0;
    for (size_t c = 0; c < classes.size(); ++c) {
      double cs = 1.0;
      for (int b : classes[c].decoration) cs = cs * basis.scale[b];
      double corr = (double)C[c] * cs / ((double)n() * (double)classes[c].multiplicity);
      E += V[c] * corr;
    }
    return E * (double)n();
  }

  // mu . (N dx) for o -> o2, composition axes: x_i = n(species i+1) / N_uc
  double mu_dot_Ndx(const std::vector<double>& mu, int o, int o2) const {
    double r = 0.0;
    for (size_t i = 0; i < mu.size(); ++i) {
      double d = (o2 == (int)i + 1 ? 1.0 : 0.0) - (o == (int)i + 1 ? 1.0 : 0.0);
      r += mu[i] * d;
    }
    return r;
  }
};

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers: as easy
// as 1, 2, 3"): round multipliers 0xD2511F53, 0xCD9E8D57; Weyl key increments
// 0x9E3779B9, 0xBB67AE85.
inline std::array<uint32_t, 4> philox4x32_10(std::array<uint32_t, 4> c, std::array<uint32_t, 2> k) {
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k[0] += 0x9E3779B9u;
      k[1] += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c = {hi1 ^ c[1] ^ k[0], lo1, hi0 ^ c[3] ^ k[1], lo0};
  }
  return c;
}

constexpr uint32_t SWEEP_TAG = 0x4D434753u;  // stream tag for the SGC sweep

struct ColoredRun {
  std::vector<std::vector<long long>> corr;  // [pass][class] after each pass
  std::vector<long long> n_accept;           // [pass]
};

// Philox block of a site and the word of it the site uses.  Binary basis with L0 = 4Q:
// the four sites i0 + tQ (0 <= i0 < Q) of a row share the block with counter word
// q = i0 + L0 (j + L1 k) and site i0 + tQ takes word t.  Otherwise (ternary basis, or L0
// not a multiple of 4) site l has its own block (counter word l) and takes words 0
// (acceptance) and 1 (choice of the new species).
inline void sweep_counter(const CESupercell& S, long l, uint32_t* q, int* word) {
  if (S.basis.n_species == 2 && S.L0 % 4 == 0) {
    const long Q = S.L0 / 4, i = l % S.L0;
    *q = (uint32_t)(l - (i / Q) * Q);
    *word = (int)(i / Q);
  } else {
    *q = (uint32_t)l;
    *word = 0;
  }
}

// Coloured semi-grand canonical sweep: pass p, colour c = 0..nc-1, every site of colour c
// visited once (order irrelevant: same-colour sites share no cluster).  Proposal:
// binary o -> 1-o; ternary o -> (o + 1 + (x1 >> 31)) % 3.  Acceptance (metropolis.hh:26-35
// with u = x0 * 2^-32, x0 the site's word of its Philox block): dE < 0 or u < exp(-beta dE).
inline ColoredRun colored_sweep(const CESupercell& S, int* occ, double T,
                                const std::vector<double>& mu, uint64_t seed, uint32_t chain,
                                const std::vector<int>& color, int n_colors, long pass0,
                                long n_passes) {
  ColoredRun R;
  double beta = 1.0 / (KB * T);
  std::vector<std::vector<long>> by_color(n_colors);
  for (long l = 0; l < S.n(); ++l) by_color[color[l]].push_back(l);
  std::array<uint32_t, 2> key{(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (long p = pass0; p < pass0 + n_passes; ++p) {
    long long nacc = 0;
    for (int c = 0; c < n_colors; ++c) {
      for (long l : by_color[c]) {
        uint32_t q;
        int word;
        sweep_counter(S, l, &q, &word);
        auto x = philox4x32_10({q, (uint32_t)p, chain, SWEEP_TAG}, key);
        const uint32_t x0 = x[word];
        int o = occ[l];
        int o2 = (S.basis.n_species == 2) ? 1 - o : (o + 1 + (int)(x[1] >> 31)) % 3;
        double dE = S.delta_formation(occ, l, o2) - S.mu_dot_Ndx(mu, o, o2);
        bool acc;
        if (dE < 0.0) {
          acc = true;
        } else {
          double u = (double)x0 * (1.0 / 4294967296.0);
          acc = u < std::exp(-dE * beta);
        }
        if (acc) {
          occ[l] = o2;
          ++nacc;
        }
      }
    }
    R.corr.push_back(S.int_corr(occ));
    R.n_accept.push_back(nacc);
  }
  return R;
}

constexpr uint32_t CANON_TAG = 0x4D434343u;    // acceptance draws of the canonical sweep
constexpr uint32_t CANON_D_TAG = 0x4D434344u;  // matching offsets of the canonical sweep

// Coloured canonical sweep: pass p uses colouring A (p even) or B (p odd); colour c = 0..n-1
// of it; the class's sites s_0, s_1, ..., s_{n-1} in list order; matching offset
// d = (x * n) >> 32 with x word 0 of Philox(c, p, chain, CANON_D_TAG); positions k and
// k2 = (d - k) mod n with k < k2 form a pair (i, j) = (s_k, s_k2); a pair of different
// occupants is exchanged by Metropolis (metropolis.hh:26-35) with u = word 0 of
// Philox(i, p, chain, CANON_TAG) * 2^-32 and dE the formation-energy change of the swap
// (the two sites share no cluster, so dE = dE_i + dE_j).  The swap is the canonical event of
// OccEventProposal.hh:108-237 with its pair chosen by the matching instead of at random.
// orderA / orderB: the sites in the order of the GPU's class lists (empty: ascending); a
// colour's class is its sites in that order.
inline ColoredRun colored_canonical_sweep(const CESupercell& S, int* occ, double T, uint64_t seed, uint32_t chain,
                                          const std::vector<int>& colA, int nA, const std::vector<int>& colB,
                                          int nB, long pass0, long n_passes, const std::vector<long>& orderA = {},
                                          const std::vector<long>& orderB = {}) {
  ColoredRun R;
  const double beta = 1.0 / (KB * T);
  std::vector<std::vector<long>> cls[2];
  cls[0].resize(nA);
  cls[1].resize(nB);
  for (long p = 0; p < S.n(); ++p) {
    const long la = orderA.empty() ? p : orderA[p], lb = orderB.empty() ? p : orderB[p];
    cls[0][colA[la]].push_back(la);
    cls[1][colB[lb]].push_back(lb);
  }
  std::array<uint32_t, 2> key{(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (long p = pass0; p < pass0 + n_passes; ++p) {
    long long nacc = 0;
    const auto& by_color = cls[p & 1];
    for (int c = 0; c < (int)by_color.size(); ++c) {
      const auto& site = by_color[c];
      const long n = (long)site.size();
      if (n < 2) continue;
      const auto xd = philox4x32_10({(uint32_t)c, (uint32_t)p, chain, CANON_D_TAG}, key);
      const long d = (long)(((uint64_t)xd[0] * (uint64_t)n) >> 32);
      for (long k = 0; k < n; ++k) {
        long k2 = d - k;
        if (k2 < 0) k2 += n;
        if (!(k < k2)) continue;
        const long i = site[k], j = site[k2];
        const int oi = occ[i], oj = occ[j];
        if (oi == oj) continue;
        const auto x = philox4x32_10({(uint32_t)i, (uint32_t)p, chain, CANON_TAG}, key);
        const double dE = S.delta_formation(occ, i, oj) + S.delta_formation(occ, j, oi);
        bool acc;
        if (dE < 0.0) {
          acc = true;
        } else {
          const double u = (double)x[0] * (1.0 / 4294967296.0);
          acc = u < std::exp(-dE * beta);
        }
        if (acc) {
          occ[i] = oj;
          occ[j] = oi;
          ++nacc;
        }
      }
    }
    R.corr.push_back(S.int_corr(occ));
    R.n_accept.push_back(nacc);
  }
  return R;
}

}  // namespace oracle

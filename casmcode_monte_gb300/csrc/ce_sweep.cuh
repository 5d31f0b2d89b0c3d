// Graph-coloured semi-grand canonical Metropolis sweep over FCC cluster-expansion
// Hamiltonians (device code, templated on a generated basis set).
//
// Correspondence with the reference loop (basic_occupation_metropolis.hh:381-421 and
// metropolis.hh:26-35): every site is proposed once per pass (colour by colour, so
// that same-colour sites share no cluster and are updated concurrently); the change
// of semi-grand canonical energy is dE = dE_f - mu.(N dx) (basic_semigrand_canonical.hh:
// 178-192); a proposal is accepted if dE < 0 or u < exp(-beta dE).  Random numbers are
// Philox4x32-10 keyed by the chain's seed with counter (q, pass, chain, tag): for the
// binary basis with L0 = 4Q the four sites i0 + tQ of a row share q = i0 + L0 (j + L1 k)
// and take words t = 0..3; otherwise q = l (words 0 and 1).  A trajectory is a pure
// function of (seed, chain, initial state), independent of the thread mapping.
//
// Layout: a chain is owned by a cluster of S CTAs; CTA r holds planes
// [k0(r), k0(r) + nk(r)) of the L0 x L1 x L2 supercell (l = i + L0*(j + L1*k)) plus a
// HALO-plane border in k and a HALO-column border in i and j, as int8 codes in shared
// memory (padded index (i+2) + PX*((j+2) + PY*(k_local+2))).  Neighbour loads are
// constant offsets from the site's padded index.  An accepted flip writes the site and
// its periodic copies (own padding and, through distributed shared memory, the halo
// planes of the neighbouring CTAs).  Phases are separated by cluster barriers
// (release/acquire).
//
// Energies: the generated feature function yields integer local sums F[k]; the FP32
// fast path computes dE32 = qscale * sum_b dpsi_b * (sum_k wq[k] F[k]) - dmu, the sum an
// exact integer of quantised weights (any split of it gives the same value).  A proposal whose
// FP32 decision could differ from the FP64 one (|dE32| within the rounding bound, or u
// within the relative bound of exp(-beta dE)) is re-decided exactly in FP64.  Accepted
// changes of the integer correlation sums are accumulated exactly (int32 per thread per
// pass, int64 per chain per pass), so per-pass energies carry no drift.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "mg_common.cuh"

namespace mg {

namespace cg = cooperative_groups;

constexpr int CE_MAX_SPECIES = 3;
constexpr int CE_MAX_MAP = 16;  // chains of one mapped launch of the warp-specialised kernel

struct CeChainParams {
  double beta;
  float beta_log2e;
  float dtol;  // bound on |dE32 - dE64|
  float eps;   // relative bound on the fast-path acceptance probability
  uint32_t key0, key1;
  uint32_t chain_id;
  double dmu64[CE_MAX_SPECIES * CE_MAX_SPECIES];  // mu . N dx for o -> o2
  float dmu32[CE_MAX_SPECIES * CE_MAX_SPECIES];
  double mu[CE_MAX_SPECIES - 1];  // exchange potentials (for energy samples)
};

// per-class energy weights w_f = V_f / M_f * C_f (E_f per supercell = sum_f w_f IntCorr_f)
template <int NCLASS>
struct CeWeightsClass {
  double w[NCLASS];
};

// Energy weights: FP64 for the exact decision; quantised integers wq[k] = round(w[k] * 2^s)
// for the fast path, whose change of energy sum_b dpsi_b * sum_k wq[k] F[k] is an exact
// int32 (s chosen so it cannot overflow) scaled by qscale = 2^-s.
// Ternary basis: the same quantised energy sums from monomial counts of the neighbours'
// indicators (the word layouts' counts_quad): sum_k wq[k] F_k of basis b = cgc[b] +
// sum_j cw[b][j] M_j (int32, exact modulo 2^32).  Unused for the binary basis.
constexpr int kMaxCounts = 32;

template <int NFEAT>
struct CeWeights {
  int wq[NFEAT];
  float qscale;
  double w64[NFEAT];
  int cw[2][kMaxCounts];
  int cgc[2];
};

struct CeGeometry {
  int L0, L1, L2;
  int S;  // CTAs per chain; CTA r owns nk(r) = L2/S (+1 for r < L2%S) planes
  int PX, PY, PZ;  // padded dims; PZ = max planes per CTA + 2 * HALO
  int n_colors;
  const int* color_start;    // [S][n_colors + 1]
  const uint32_t* entries;   // padded index | flags << 24
  const uint32_t* site_l;    // global linear site index per entry
};

// slot layout of the per-pass outputs: 0 = accepted proposals, f = change of the
// integer correlation sum of class f (1..NCLASS-1), NCLASS = proposals re-decided in
// FP64, NCLASS+1 = FP32 decisions that differ from FP64 (FP32 mode only)
template <int NCLASS>
struct CeSlots {
  static constexpr int N = NCLASS + 2;
};

template <int NFEAT>
struct CeSweepArgs {
  CeGeometry g;
  CeWeights<NFEAT> w;
  const CeChainParams* cp;  // [chain]
  int8_t* occ;              // [chain][N] occupant indices
  long long pass0;
  int n_passes;
  int n_chains;
  int precision;   // 0: FP64 decisions; 1: FP32 decisions (flips counted)
  long long* out;  // [n_passes][n_chains][NSLOT]
};

struct SmemLoader {
  const int8_t* p;
  int PX, PXY;
  __device__ __forceinline__ int operator()(int di, int dj, int dk) const {
    return p[di + dj * PX + dk * PXY];
  }
};

__device__ __forceinline__ float fast_exp2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// split cluster barrier: arrive (release the CTA's shared and distributed-shared writes),
// then wait (acquire the other CTAs' writes)
__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Metropolis decision of one proposal o -> o2 from its integer local features, in two
// parts: fast() is the branch-free FP32 decision from the exact integer change dEq and
// says whether it is ambiguous (|dE32| within the quantisation and rounding bound, or u
// within the relative bound of exp(-beta dE)); exact() takes the FP64 decision of an
// ambiguous proposal, counts it in acc[NCLASS] and, in FP32 mode, counts a flipped
// decision in acc[NCLASS+1] (the FP32 decision stands there).  Fi(k) returns F[k].
template <class B>
struct MetropolisRule {
  static constexpr int NF = B::NFEAT;
  static constexpr int NC = B::NCLASS;
  static constexpr int NS = B::NSPECIES;
  static constexpr int NSLOT = CeSlots<NC>::N;
  const float* dmu32;  // shared memory [NS*NS]
  const double* dmu64;
  const CeWeights<NF>* w;
  double beta;
  float beta_log2e, dtol, eps;
  int precision;

  // exact integer change of energy sum_b dpsi_b * sum_k wq[k] F[k] (F[k] = Fi(k))
  template <class FI>
  __device__ __forceinline__ int dEq(const int (&dpsi)[B::NFUNC], const FI& Fi) const {
    int G[B::NFUNC];
#pragma unroll
    for (int b = 0; b < B::NFUNC; ++b) G[b] = 0;
#pragma unroll
    for (int k = 0; k < NF; ++k) G[B::feat_b(k)] += w->wq[k] * Fi(k);
    int d = 0;
#pragma unroll
    for (int b = 0; b < B::NFUNC; ++b) d += dpsi[b] * G[b];
    return d;
  }

  // The band around P = 2^a, a = -beta log2(e) dE32, holds every u whose FP64 decision
  // could differ: relative half-width eps (per chain: the quantisation error and the
  // rounding of mu.N dx through exp, the ex2.approx error, the roundings of u and of the
  // band edges) plus 2e-7 |a| (the FP32 roundings of dE32, of order 2^-23 |dE32|, through
  // exp, and the rounding of a itself).
  __device__ __forceinline__ bool fast(int o, int o2, int dEq, uint32_t x0, bool& amb) const {
    const float dE32 = fmaf((float)dEq, w->qscale, -dmu32[o * NS + o2]);
    const float u32 = __uint2float_rn(x0) * 2.3283064365386963e-10f;
    const float a = -dE32 * beta_log2e;
    const float P = fast_exp2(a);
    const float e = fmaf(fabsf(a), 2.0e-7f, eps);
    const bool band = !(u32 < P * (1.f - e)) && !(u32 > P * (1.f + e));
    amb = !(dE32 < -dtol) && ((dE32 <= dtol) || (x0 == 0u) || band);
    return (dE32 < 0.f) || (u32 < P);
  }

  template <class FI>
  __device__ __forceinline__ bool exact(int o, int o2, const int (&dpsi)[B::NFUNC], const FI& Fi, uint32_t x0,
                                     bool acc32, int (&acc)[NSLOT]) const {
    // dE64 = sum_b dpsi_b * (sum_k w64[k] F[k]) - dmu
    double G64[B::NFUNC];
#pragma unroll
    for (int b = 0; b < B::NFUNC; ++b) G64[b] = 0.0;
#pragma unroll
    for (int k = 0; k < NF; ++k) G64[B::feat_b(k)] = __fma_rn(w->w64[k], (double)Fi(k), G64[B::feat_b(k)]);
    double dE = -dmu64[o * NS + o2];
#pragma unroll
    for (int b = 0; b < B::NFUNC; ++b) dE = __fma_rn((double)dpsi[b], G64[b], dE);
    bool acc64;
    if (dE < 0.0) {
      acc64 = true;
    } else {
      const double u = __dmul_rn((double)x0, 2.3283064365386962890625e-10);
      acc64 = u < exp(__dmul_rn(-dE, beta));
    }
    acc[NC] += 1;
    if (precision == 0) return acc64;
    if (acc64 != acc32) acc[NC + 1] += 1;
    return acc32;
  }

  template <class FI>
  __device__ __forceinline__ bool operator()(int o, int o2, const int (&dpsi)[B::NFUNC], const FI& Fi, uint32_t x0,
                                             int (&acc)[NSLOT]) const {
    bool amb;
    const bool acc32 = fast(o, o2, dEq(dpsi, Fi), x0, amb);
    if (amb) return exact(o, o2, dpsi, Fi, x0, acc32, acc);
    return acc32;
  }
};

template <class B>
__device__ __noinline__ int tern_exact(const MetropolisRule<B>& rule, int o, int o2, int dpsi0, int dpsi1,
                                       const uint32_t* M, int shift, uint32_t x0, bool acc32);

// word `w` (0..3) of a Philox block
__device__ __forceinline__ uint32_t philox_word(const U32x4& x, uint32_t w) {
  return w == 0u ? x.x : (w == 1u ? x.y : (w == 2u ? x.z : x.w));
}

// Neighbours of four byte-layout sites (any four of one colour) packed into words, byte t
// from site t, as occupants 0..2 (codes o - 1 = 0xFF, 0x00, 0x01 plus one per byte, without
// carries between bytes): the input of counts_quad for four sites at once
template <class B>
struct GatherWordLoader {
  const int8_t* s;
  int i0, i1, i2, i3;  // padded indices of the four sites
  int PX, PXY;
  __device__ __forceinline__ uint32_t operator()(int di, int dj, int dk) const {
    const int off = di + dj * PX + dk * PXY;
    const uint32_t a = (uint8_t)s[i0 + off], b = (uint8_t)s[i1 + off], c = (uint8_t)s[i2 + off],
                   d = (uint8_t)s[i3 + off];
    const uint32_t w = __byte_perm(__byte_perm(a, b, 0x0040), __byte_perm(c, d, 0x0040), 0x5410);
    static_assert(B::code_of_occ(0) == -1 && B::code_of_occ(2) == 1, "ternary codes are o - 1");
    return ((w & 0x7F7F7F7Fu) + 0x01010101u) ^ (w & 0x80808080u);
  }
};

// Per-CTA context of the site update: shared-memory lattice and its periodic copies,
// chain constants and the FP32/FP64 decision rule.  Shared by the cluster sweep kernel
// and the persistent pool kernel.
template <class B>
struct SiteSweeper {
  static constexpr int NF = B::NFEAT;
  static constexpr int NC = B::NCLASS;
  static constexpr int NS = B::NSPECIES;
  static constexpr int NSLOT = CeSlots<NC>::N;
  int8_t* s;       // own slab (padded)
  int8_t* s_prev;  // previous CTA's slab (distributed shared memory; == s for one CTA)
  int8_t* s_next;  // next CTA's slab
  int PX, PXY;
  int dI, dJ, dKp, dKn;  // offsets of the periodic / halo copies
  const float* dmu32;    // shared memory [NS*NS]
  const double* dmu64;
  const CeWeights<NF>* w;
  double beta;
  float beta_log2e, dtol, eps;
  int precision;

  // the site's occupant and its integer local features
  __device__ __forceinline__ void gather(uint32_t ent, int& o, int (&F)[NF]) const {
    const int8_t* p = s + (int)(ent & 0xFFFFFFu);
    o = B::occ_of_code(*p);
    B::features(SmemLoader{p, PX, PXY}, F);
  }

  // Metropolis decision for the proposal drawn from (x0, x1); on acceptance write the
  // site and its copies and add the changes of the integer correlation sums to acc.
  __device__ __forceinline__ void decide(uint32_t ent, uint32_t x0, uint32_t x1, int o, const int (&F)[NF],
                                         int (&acc)[NSLOT]) const {
    int o2;
    if (NS == 2)
      o2 = 1 - o;
    else
      o2 = (o + 1 + (int)(x1 >> 31)) % 3;
    int dpsi[B::NFUNC];
#pragma unroll
    for (int b = 0; b < B::NFUNC; ++b) dpsi[b] = B::psi(b, o2) - B::psi(b, o);
    const MetropolisRule<B> rule{dmu32, dmu64, w, beta, beta_log2e, dtol, eps, precision};
    const bool accept = rule(o, o2, dpsi, [&](int k) { return F[k]; }, x0, acc);
    if (accept) {
      store(ent, B::code_of_occ(o2));
      acc[0] += 1;
#pragma unroll
      for (int k = 0; k < NF; ++k) acc[B::feat_class(k)] += dpsi[B::feat_b(k)] * F[k];
    }
  }

  // Ternary basis, four sites of one colour at once (entries ent[t], Philox counter words
  // sl[t]; sites t >= n are absent and only repeat site 0's loads): the counts of the four
  // sites byte-parallel from gathered neighbour words, then per site the proposal, energy
  // sums (equal to sum_k wq[k] F_k), FP32 rule and FP64 re-decision of decide(), so every
  // decision and the trajectory are those of the one-site update; the correlation changes of
  // the accepted sites as byte dot products of the counts with the packed dpsi.
  // (entries and counter words of site t at index e[t] of `entries` / `site_l`; read
  // again after the counts rather than held through them)
  __device__ __forceinline__ void update_gathered(const uint32_t* entries, const uint32_t* site_l, const int (&e)[4],
                                                  int n, uint32_t pass, uint32_t chain_id, uint32_t key0,
                                                  uint32_t key1, int (&acc)[NSLOT]) const {
    constexpr int NJ = B::NCOUNT;
    static_assert(NJ <= kMaxCounts, "count weights");
    uint32_t v;
    uint32_t M[NJ];
    {
      const int i0 = (int)(__ldg(entries + e[0]) & 0xFFFFFFu);
      const int i1 = n > 1 ? (int)(__ldg(entries + e[1]) & 0xFFFFFFu) : i0;
      const int i2 = n > 2 ? (int)(__ldg(entries + e[2]) & 0xFFFFFFu) : i0;
      const int i3 = n > 3 ? (int)(__ldg(entries + e[3]) & 0xFFFFFFu) : i0;
      const GatherWordLoader<B> ld{s, i0, i1, i2, i3, PX, PXY};
      v = ld(0, 0, 0);
      B::counts_quad(ld, M);
    }
    const MetropolisRule<B> rule{dmu32, dmu64, w, beta, beta_log2e, dtol, eps, precision};
    uint32_t sg0 = 0u, sg1 = 0u;
    int n_acc = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      if (t >= n) break;
      const uint32_t ent = __ldg(entries + e[t]);
      const U32x4 x = philox4x32_10(U32x4{__ldg(site_l + e[t]), pass, chain_id, SWEEP_TAG}, key0, key1);
      const uint32_t x0 = philox_word(x, ent >> 30);
      const int o = (int)((v >> (8 * t)) & 0xFFu);
      const int o2 = (o + 1 + (int)(x.y >> 31)) % 3;
      const int dpsi0 = B::psi(0, o2) - B::psi(0, o), dpsi1 = B::psi(1, o2) - B::psi(1, o);
      int G0 = w->cgc[0], G1 = w->cgc[1];
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const int m = (int)((M[j] >> (8 * t)) & 0xFFu);
        G0 += w->cw[0][j] * m;
        G1 += w->cw[1][j] * m;
      }
      bool amb;
      bool a = rule.fast(o, o2, dpsi0 * G0 + dpsi1 * G1, x0, amb);
      if (amb) {
        uint32_t Mc[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) Mc[j] = M[j];
        const int r = tern_exact<B>(rule, o, o2, dpsi0, dpsi1, Mc, 8 * t, x0, a);
        a = (r & 1) != 0;
        acc[NC] += 1;
        acc[NC + 1] += (r >> 1) & 1;
      }
      if (a) {
        store(ent, B::code_of_occ(o2));
        sg0 |= (uint32_t)(dpsi0 & 0xFF) << (8 * t);
        sg1 |= (uint32_t)(dpsi1 & 0xFF) << (8 * t);
        ++n_acc;
      }
    }
    if (n_acc) {
      acc[0] += n_acc;
      const int c0 = __dp4a((int)0x01010101, (int)sg0, 0), c1 = __dp4a((int)0x01010101, (int)sg1, 0);
#pragma unroll
      for (int k = 0; k < NF; ++k)
        if (B::tq_const(k) != 0) acc[B::feat_class(k)] += B::tq_const(k) * (B::feat_b(k) == 0 ? c0 : c1);
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const int d0 = __dp4a((int)M[j], (int)sg0, 0), d1 = __dp4a((int)M[j], (int)sg1, 0);
#pragma unroll
        for (int k = 0; k < NF; ++k)
          if (B::tq_coef(k, j) != 0) acc[B::feat_class(k)] += B::tq_coef(k, j) * (B::feat_b(k) == 0 ? d0 : d1);
      }
    }
  }

  // write code c2 at the entry's site and at its periodic copies (own padding and, through
  // distributed shared memory, the halo planes of the neighbouring CTAs)
  __device__ __forceinline__ void store(uint32_t ent, int8_t c2) const {
    const int pidx = (int)(ent & 0xFFFFFFu);
    const uint32_t flags = ent >> 24;
    const int oi = (flags & 1u) ? dI : ((flags & 2u) ? -dI : 0);
    const int oj = (flags & 4u) ? dJ : ((flags & 8u) ? -dJ : 0);
    s[pidx] = c2;
    if (oi) s[pidx + oi] = c2;
    if (oj) s[pidx + oj] = c2;
    if (oi && oj) s[pidx + oi + oj] = c2;
    if (flags & 16u) {
      int8_t* r = s_prev + pidx + dKp;
      r[0] = c2;
      if (oi) r[oi] = c2;
      if (oj) r[oj] = c2;
      if (oi && oj) r[oi + oj] = c2;
    }
    if (flags & 32u) {
      int8_t* r = s_next + pidx - dKn;
      r[0] = c2;
      if (oi) r[oi] = c2;
      if (oj) r[oj] = c2;
      if (oi && oj) r[oi + oj] = c2;
    }
  }
};

// Philox words of the first PRE sites of a thread in one colour phase, drawn ahead of
// the phase (they depend on (site, pass, chain) only, not on the lattice).  The list
// holds each site's counter word and, in the entry's top two bits, the word it takes.
template <int PRE>
struct PhasePrefetch {
  uint32_t ent[PRE], x0[PRE], x1[PRE];

  template <int NT>
  __device__ __forceinline__ void prepare(const int* cstart, int c, const uint32_t* entries,
                                          const uint32_t* site_l, uint32_t pass, uint32_t chain_id,
                                          uint32_t key0, uint32_t key1) {
    const int eb = cstart[c] + threadIdx.x, ee = cstart[c + 1];
#pragma unroll
    for (int q = 0; q < PRE; ++q) {
      const int e = eb + q * NT;
      if (e < ee) {
        ent[q] = __ldg(entries + e);
        const U32x4 x = philox4x32_10(U32x4{__ldg(site_l + e), pass, chain_id, SWEEP_TAG}, key0, key1);
        x0[q] = philox_word(x, ent[q] >> 30);
        x1[q] = x.y;
      }
    }
  }
};

// Site grouping of the ternary byte-layout sweep: one site per thread and step, four, or
// chosen per phase (four when the phase has more than 1.5 sites per thread).  The host picks
// one or four per launch of a chain batch from its sites per CTA and colour (the two paths
// compiled together spill more registers); the pool kernels, whose chains differ in shape,
// choose per phase.
constexpr int kSitesOne = 1, kSitesFour = 2, kSitesPerPhase = 0;

// One colour phase of one CTA: the prefetched sites, then any further sites inline.
template <class B, int NT, int PRE, int GROUP = kSitesPerPhase>
__device__ __forceinline__ void sweep_phase(const SiteSweeper<B>& sw, const PhasePrefetch<PRE>& pf,
                                            const int* cstart, int c, const uint32_t* entries,
                                            const uint32_t* site_l, uint32_t pass, uint32_t chain_id,
                                            uint32_t key0, uint32_t key1, int (&acc)[SiteSweeper<B>::NSLOT]) {
  const int e0 = cstart[c] + threadIdx.x, e_end = cstart[c + 1];
  // ternary basis, four sites per thread and step (entries q, q + T, q + 2T, q + 3T of the
  // phase's list, T = ceil(n / 4), so the lanes of a warp still read consecutive entries);
  // with few sites per thread one site per thread and step is faster (its dependent chain is
  // shorter): GB300, 8 ternary chains of 64^3 (3.6 sites per thread and colour) 259 -> 167 us
  // per pass with four, 8 of 30^3 (0.4 per thread) 58 us with one against 109 with four
  if (B::NSPECIES == 3 && GROUP != kSitesOne &&
      (GROUP == kSitesFour || 2 * (e_end - cstart[c]) > 3 * NT)) {
    const int base = cstart[c], n_e = e_end - base, T = (n_e + 3) >> 2;
#pragma unroll 1
    for (int q = threadIdx.x; q < T; q += NT) {
      int e[4];
      int n = 0;
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        e[t] = base + q + t * T;
        if (q + t * T < n_e) n = t + 1;
      }
      if constexpr (B::NSPECIES == 3) sw.update_gathered(entries, site_l, e, n, pass, chain_id, key0, key1, acc);
    }
  } else if constexpr (B::NSPECIES != 3 || GROUP != kSitesFour) {
#pragma unroll
    for (int q = 0; q < PRE; ++q)
      if (e0 + q * NT < e_end) {
        int o;
        int F[B::NFEAT];
        sw.gather(pf.ent[q], o, F);
        sw.decide(pf.ent[q], pf.x0[q], pf.x1[q], o, F, acc);
      }
#pragma unroll 1
    for (int e = e0 + PRE * NT; e < e_end; e += NT) {
      const U32x4 x = philox4x32_10(U32x4{__ldg(site_l + e), pass, chain_id, SWEEP_TAG}, key0, key1);
      const uint32_t ent = __ldg(entries + e);
      int o;
      int F[B::NFEAT];
      sw.gather(ent, o, F);
      sw.decide(ent, philox_word(x, ent >> 30), x.y, o, F, acc);
    }
  }
}

template <int NS>
__device__ __forceinline__ void load_dmu(const CeChainParams* cp, float* dmu32, double* dmu64) {
  if (threadIdx.x < NS * NS) {
    dmu32[threadIdx.x] = cp->dmu32[threadIdx.x];
    dmu64[threadIdx.x] = cp->dmu64[threadIdx.x];
  }
}

template <class B, int NT, int GROUP = kSitesOne>
__global__ void __launch_bounds__(NT, 1) ce_sweep_kernel(const __grid_constant__ CeSweepArgs<B::NFEAT> A) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  constexpr int PRE = (NS == 2) ? 3 : 1;
  extern __shared__ __align__(16) int8_t s[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];

  const CeGeometry& g = A.g;
  const int S = g.S;
  const int chain = blockIdx.x / S;
  int rank = 0;
  cg::cluster_group cluster = cg::this_cluster();
  if (S > 1) rank = (int)cluster.block_rank();
  auto barrier = [&]() {
    if (S > 1)
      cluster.sync();
    else
      __syncthreads();
  };

  const int PX = g.PX, PY = g.PY, PXY = PX * PY;
  const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
  const int nkq = L2 / S, nkr = L2 % S;
  const int nk = nkq + (rank < nkr ? 1 : 0);
  const int k0 = rank * nkq + (rank < nkr ? rank : nkr);
  const int rprev = (rank + S - 1) % S;
  const int nk_prev = nkq + (rprev < nkr ? 1 : 0);
  const long long N = (long long)L0 * L1 * L2;
  int8_t* gocc = A.occ + (size_t)chain * N;

  // ---- load slab + borders
  for (int idx = threadIdx.x; idx < PXY * (nk + 2 * B::HALO); idx += NT) {
    const int ip = idx % PX, jp = (idx / PX) % PY, kp = idx / PXY;
    int i = ip - B::HALO, j = jp - B::HALO, k = k0 + kp - B::HALO;
    i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
    j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
    k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
    s[idx] = B::code_of_occ(gocc[i + (long long)L0 * (j + (long long)L1 * k)]);
  }
  if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;

  const CeChainParams* cpg = A.cp + chain;
  load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
  const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
  const int* cstart = g.color_start + rank * (g.n_colors + 1);

  // periodic copies: +-L0 in i, +-L1 rows in j; a plane kl < HALO is also the upper
  // halo of the previous CTA (at kl + nk_prev + HALO), a plane kl >= nk - HALO the
  // lower halo of the next CTA (at kl - nk + HALO)
  SiteSweeper<B> sw;
  sw.s = s;
  sw.s_prev = s;
  sw.s_next = s;
  if (S > 1) {
    sw.s_prev = cluster.map_shared_rank(s, (unsigned)rprev);
    sw.s_next = cluster.map_shared_rank(s, (unsigned)((rank + 1) % S));
  }
  sw.PX = PX;
  sw.PXY = PXY;
  sw.dI = L0;
  sw.dJ = L1 * PX;
  sw.dKp = nk_prev * PXY;
  sw.dKn = nk * PXY;
  sw.dmu32 = dmu32_sm;
  sw.dmu64 = dmu64_sm;
  sw.w = &A.w;
  sw.beta = cpg->beta;
  sw.beta_log2e = cpg->beta_log2e;
  sw.dtol = cpg->dtol;
  sw.eps = cpg->eps;
  sw.precision = A.precision;
  const int lane = threadIdx.x & 31;
  int acc[NSLOT];
#pragma unroll
  for (int q = 0; q < NSLOT; ++q) acc[q] = 0;

  PhasePrefetch<PRE> pf;
  pf.template prepare<NT>(cstart, 0, g.entries, g.site_l, (uint32_t)A.pass0, chain_id, key0, key1);
  barrier();

#pragma unroll 1
  for (int pass = 0; pass < A.n_passes; ++pass) {
    const uint32_t pass_g = (uint32_t)(A.pass0 + pass);
#pragma unroll 1
    for (int c = 0; c < g.n_colors; ++c) {
      sweep_phase<B, NT, PRE, GROUP>(sw, pf, cstart, c, g.entries, g.site_l, pass_g, chain_id, key0, key1, acc);
      const bool last = (c + 1 == g.n_colors);
      if (S > 1) {
        // arrive, draw the next phase's random numbers while others finish, then wait
        cluster_arrive_release();
        pf.template prepare<NT>(cstart, last ? 0 : c + 1, g.entries, g.site_l, last ? pass_g + 1 : pass_g,
                                chain_id, key0, key1);
        cluster_wait_acquire();
      } else {
        pf.template prepare<NT>(cstart, last ? 0 : c + 1, g.entries, g.site_l, last ? pass_g + 1 : pass_g,
                                chain_id, key0, key1);
        __syncthreads();
      }
      if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
        // flush the previous pass (all warps added to it before this barrier)
        int* buf = acc_sm[(pass - 1) & 1];
        const int v = buf[threadIdx.x];
        buf[threadIdx.x] = 0;
        if (v)
          atomicAdd(reinterpret_cast<unsigned long long*>(
                        A.out + ((size_t)(pass - 1) * A.n_chains + chain) * NSLOT + threadIdx.x),
                    (unsigned long long)(long long)v);
      }
    }
    // per-warp reduction of this pass's accumulators into shared memory
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) {
      const int v = warp_sum(acc[q]);
      if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
      acc[q] = 0;
    }
  }
  barrier();
  if (A.n_passes > 0 && threadIdx.x < NSLOT) {
    const int pl = A.n_passes - 1;
    int* buf = acc_sm[pl & 1];
    const int v = buf[threadIdx.x];
    if (v)
      atomicAdd(reinterpret_cast<unsigned long long*>(A.out + ((size_t)pl * A.n_chains + chain) * NSLOT + threadIdx.x),
                (unsigned long long)(long long)v);
  }
  // ---- write back own planes
  for (int idx = threadIdx.x; idx < L0 * L1 * nk; idx += NT) {
    const int i = idx % L0, j = (idx / L0) % L1, kl = idx / (L0 * L1);
    const int pidx = (i + B::HALO) + PX * ((j + B::HALO) + PY * (kl + B::HALO));
    gocc[i + (long long)L0 * (j + (long long)L1 * (k0 + kl))] = (int8_t)B::occ_of_code(s[pidx]);
  }
  barrier();
}

// ---- word layout (binary occupation basis): four sites per 32-bit word
//
// A supercell row (fixed j, k) of L0 = 4Q sites is held as Q words; word w in [0, Q)
// holds the sites i = w + tQ in byte t (t = 0..3).  The padded row has words
// w in [-2, Q + 2): words -2, -1 are words Q-2, Q-1 rotated left by one byte and words
// Q, Q+1 are words 0, 1 rotated right by one byte, so that byte t of padded word w is
// always site (w + tQ) mod L0.  A neighbour offset (di, dj, dk) of the four sites of a
// word is then the word at constant offset di + dj*RS + dk*RS*RY, with the four
// neighbours in matching bytes.  With a colouring in which colour(i + Q) = colour(i), a
// word's four sites share a colour and are proposed together: the features of all four
// come out of one pass of byte-parallel integer code, the four decisions are taken one
// by one (same random numbers, same arithmetic as the per-site kernel, so trajectories
// are identical), and accepted flips are written back as one word.
// Row slabs of the word layout.  With rows numbered R = j + L1 k, CTA r of S owns the
// rows [R_r, R_r+1): balanced, R_r = floor(r L1 L2 / S), so that every CTA proposes the
// same number of words (to within one row) whatever S divides; or, where balanced slabs
// are too thin for the halo, whole planes (R_r = L1 (r floor(L2/S) + min(r, L2 mod S))).
// A slab's shared-memory window holds the nk planes its rows touch, from plane kb, plus
// HALO planes on each side; the rows of the window it does not own belong to the
// previous or the next CTA, which write their updates into it.  A word at local offset pw
// of CTA r lies at pw + dkp RSY in the previous CTA's window and at pw - dkn RSY in the
// next CTA's (plane offsets with the periodic wrap of the first and the last CTA).
struct RowSlab {
  int r0, r1;    // owned rows [r0, r1)
  int kb, nk;    // first plane touched, planes touched
  int dkp, dkn;  // plane offsets of the copies in the previous / next CTA's window
};
__host__ __device__ __forceinline__ int slab_row(int L1, int L2, int S, int r, int planes) {
  if (planes) return L1 * (r * (L2 / S) + (r < L2 % S ? r : L2 % S));
  const long long num = (long long)r * L1 * L2;
  if (num <= 0x7fffffffll) return (int)num / S;  // 32-bit division where the product fits
  return (int)(num / S);
}
__host__ __device__ __forceinline__ RowSlab row_slab(int L1, int L2, int S, int r, int planes) {
  RowSlab s;
  s.r0 = slab_row(L1, L2, S, r, planes);
  s.r1 = slab_row(L1, L2, S, r + 1, planes);
  s.kb = s.r0 / L1;
  s.nk = (s.r1 - 1) / L1 - s.kb + 1;
  const int kbp = slab_row(L1, L2, S, (r + S - 1) % S, planes) / L1;
  const int kbn = slab_row(L1, L2, S, (r + 1) % S, planes) / L1;
  s.dkp = s.kb - kbp + (r == 0 ? L2 : 0);
  s.dkn = kbn - s.kb + (r == S - 1 ? L2 : 0);
  return s;
}
// planes of the largest window (touched planes + 2 halo) and rows of the largest slab
__host__ __device__ __forceinline__ int row_window_planes(int L1, int L2, int S, int halo, int planes) {
  int m = 0;
  for (int r = 0; r < S; ++r) {
    const int n = row_slab(L1, L2, S, r, planes).nk;
    m = n > m ? n : m;
  }
  return m + 2 * halo;
}
__host__ __device__ __forceinline__ int row_slab_max_rows(int L1, int L2, int S, int planes) {
  int m = 0;
  for (int r = 0; r < S; ++r) {
    const int n = slab_row(L1, L2, S, r + 1, planes) - slab_row(L1, L2, S, r, planes);
    m = n > m ? n : m;
  }
  return m;
}

// 4 x 4 byte transpose: byte t of out[m] = byte m of in[t] (its own inverse)
__device__ __forceinline__ void transpose4x4(const uint32_t in[4], uint32_t out[4]) {
  const uint32_t a = __byte_perm(in[0], in[1], 0x5140), b = __byte_perm(in[2], in[3], 0x5140);
  const uint32_t c = __byte_perm(in[0], in[1], 0x7362), d = __byte_perm(in[2], in[3], 0x7362);
  out[0] = __byte_perm(a, b, 0x5410);
  out[1] = __byte_perm(a, b, 0x7632);
  out[2] = __byte_perm(c, d, 0x5410);
  out[3] = __byte_perm(c, d, 0x7632);
}

// Window load when Q is a multiple of 4 and the chain's occupation is 4-byte aligned:
// word group k4 of a row (words 4 k4 .. 4 k4 + 3) is the byte transpose of the row's 32-bit
// words k4 + t Q/4, t = 0..3; the loads of U groups are issued before any is used.  Writes
// the same shared words as the byte loop below, halo copies (rotated one byte) and the
// zero padding word included.
template <int HALO>
__device__ __forceinline__ void load_word_window_x4(uint32_t* sq, const int8_t* gocc, int L1, int L2, int Q, int RS,
                                                    int RY, int kb, int nk, int tid, int nthreads) {
  constexpr int U = 4;
  const int G = Q >> 2;
  const int total = G * RY * (nk + 2 * HALO);
  const uint32_t* g32 = reinterpret_cast<const uint32_t*>(gocc);
  for (int base = tid; base < total; base += U * nthreads) {
    uint32_t v[U][4];
    int dst[U], k4s[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int idx = base + u * nthreads;
      dst[u] = -1;
      k4s[u] = 0;
      if (idx < total) {
        const int k4 = idx % G, pr = idx / G;
        const int jp = pr % RY, kp = pr / RY;
        int j = jp - HALO, k = kb + kp - HALO;
        j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
        k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
        const uint32_t* row = g32 + (long long)Q * (j + (long long)L1 * k);
#pragma unroll
        for (int t = 0; t < 4; ++t) v[u][t] = __ldg(row + k4 + t * G);
        dst[u] = pr * RS + HALO + 4 * k4;
        k4s[u] = k4;
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (dst[u] < 0) continue;
      uint32_t w[4];
      transpose4x4(v[u], w);
      uint32_t* d = sq + dst[u];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        d[m] = w[m];
        const int wi = 4 * k4s[u] + m;
        if (wi < HALO) d[m + Q] = __funnelshift_r(w[m], w[m], 8);         // word Q + wi
        if (wi >= Q - HALO) d[m - Q] = __funnelshift_l(w[m], w[m], 8);    // word wi - Q
      }
      if (k4s[u] == G - 1 && RS > Q + 2 * HALO) d[4 + HALO] = 0u;  // padding word (w = Q + HALO)
    }
  }
}

// Load the window of a row slab into shared memory: planes kb - HALO .. kb + nk - 1 +
// HALO, each row with its periodic copies (words -HALO .. Q + HALO - 1 of a padded row of
// RS; padding words beyond are zero and never read); word w holds sites w + tQ, t = 0..3.
template <int HALO>
__device__ __forceinline__ void load_word_window(uint32_t* sq, const int8_t* gocc, int L0, int L1, int L2, int Q,
                                                 int RS, int RY, int kb, int nk, int tid, int nthreads) {
  if ((Q & 3) == 0 && HALO <= 4 && RS <= Q + 2 * HALO + 1 && (reinterpret_cast<uintptr_t>(gocc) & 3u) == 0) {
    load_word_window_x4<HALO>(sq, gocc, L1, L2, Q, RS, RY, kb, nk, tid, nthreads);
    return;
  }
  const int RSY = RS * RY;
  for (int idx = tid; idx < RSY * (nk + 2 * HALO); idx += nthreads) {
    const int wp = idx % RS, jp = (idx / RS) % RY, kp = idx / RSY;
    const int w = wp - HALO;
    uint32_t word = 0u;
    if (w < Q + HALO) {
      int j = jp - HALO, k = kb + kp - HALO;
      j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
      k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
      const int8_t* row = gocc + (long long)L0 * (j + (long long)L1 * k);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        int i = w + t * Q;
        i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
        word |= (uint32_t)(uint8_t)row[i] << (8 * t);
      }
    }
    sq[idx] = word;
  }
}

// Write the owned rows of a row slab back to the occupation array.
template <int HALO>
__device__ __forceinline__ void store_word_rows(const uint32_t* sq, int8_t* gocc, int L0, int L1, int Q, int RS,
                                                int RY, const RowSlab& sl, int tid, int nthreads) {
  if ((Q & 3) == 0 && (reinterpret_cast<uintptr_t>(gocc) & 3u) == 0) {
    // word group k4 of a row back to the row's 32-bit words k4 + t Q/4 (the same transpose)
    const int G = Q >> 2;
    uint32_t* g32 = reinterpret_cast<uint32_t*>(gocc);
    for (int idx = tid; idx < G * (sl.r1 - sl.r0); idx += nthreads) {
      const int k4 = idx % G, R = sl.r0 + idx / G;
      const int j = R % L1, k = R / L1;
      const uint32_t* s = sq + (4 * k4 + HALO) + RS * ((j + HALO) + RY * (k - sl.kb + HALO));
      const uint32_t w[4] = {s[0], s[1], s[2], s[3]};
      uint32_t v[4];
      transpose4x4(w, v);
      uint32_t* row = g32 + (long long)Q * (j + (long long)L1 * k);
#pragma unroll
      for (int t = 0; t < 4; ++t) row[k4 + t * G] = v[t];
    }
    return;
  }
  for (int idx = tid; idx < Q * (sl.r1 - sl.r0); idx += nthreads) {
    const int w = idx % Q, R = sl.r0 + idx / Q;
    const int j = R % L1, k = R / L1;
    const uint32_t word = sq[(w + HALO) + RS * ((j + HALO) + RY * (k - sl.kb + HALO))];
    int8_t* row = gocc + (long long)L0 * (j + (long long)L1 * k);
#pragma unroll
    for (int t = 0; t < 4; ++t) row[w + t * Q] = (int8_t)((word >> (8 * t)) & 0xFFu);
  }
}

struct QuadGeometry {
  int L0, L1, L2, Q;
  int S;
  int planes;  // slab kind: 0 balanced rows, 1 whole planes (row_slab)
  int RS, RY;  // padded words per row (odd: rows start in different banks), rows per plane
  int n_colors;
  const int* color_start;   // [S][n_colors + 1]
  const uint32_t* entries;  // padded word index | flags << 24
  const uint32_t* site_l;   // linear index of the word's byte-0 site
  // computed once on the host: planes of the largest window (row_window_planes with the
  // basis halo) and rows of the largest slab (row_slab_max_rows)
  int window_planes, max_rows;
};

template <int NFEAT>
struct CeQuadArgs {
  QuadGeometry g;
  CeWeights<NFEAT> w;
  const CeChainParams* cp;
  int8_t* occ;
  long long pass0;
  int n_passes;
  int n_chains;  // chains of the batch: the output's chain stride
  int precision;
  long long* out;
  // Chain map (warp-specialised kernel).  n_map == 0: the CTAs [i S, (i+1) S) sweep chain i
  // from pass pass0.  n_map > 0: they sweep chain map_chain[i], which has already advanced
  // map_pass[i] passes beyond pass0 in this call (its Philox passes and output rows start
  // there), so a call's passes can be split over launches of different cluster sizes.
  int n_map;
  int map_chain[CE_MAX_MAP];
  int map_pass[CE_MAX_MAP];
};

// neighbour words of a word at p (window strides RS, RSY); CG: the window is in global
// memory, written by other SMs between phases, so loads bypass L1 (ld.global.cg)
template <bool CG>
struct WordLoaderT {
  const uint32_t* p;
  int RS, RSY;
  __device__ __forceinline__ uint32_t operator()(int di, int dj, int dk) const {
    if constexpr (CG)
      return __ldcg(p + di + dj * RS + dk * RSY);
    else
      return p[di + dj * RS + dk * RSY];
  }
};
using WordLoader = WordLoaderT<false>;

// F[k] of one byte lane, as an int (FP64 re-decisions)
template <int NF>
struct QuadFeature {
  const uint32_t (&F)[NF];
  int shift;
  __device__ __forceinline__ int operator()(int k) const { return (int)((F[k] >> shift) & 0xFFu); }
};

template <class B>
struct QuadSweeper {
  static constexpr int NF = B::NFEAT;
  static constexpr int NC = B::NCLASS;
  static constexpr int NSLOT = CeSlots<NC>::N;
  static_assert(B::NSPECIES == 2 && B::NFUNC == 1, "word layout needs a binary occupation basis");
  uint32_t* s;
  uint32_t* s_prev;
  uint32_t* s_next;
  int RS, RSY;
  int Q, dJ, dKp, dKn;
  MetropolisRule<B> rule;

  __device__ __forceinline__ WordLoader loader(uint32_t ent) const {
    return WordLoader{s + (int)(ent & 0xFFFFFFu), RS, RSY};
  }

  // one word: features of its four sites, then finish()
  __device__ __forceinline__ void update(uint32_t ent, const uint32_t (&x0)[4], int (&acc)[NSLOT]) const {
    uint32_t F[NF];
    B::features_quad(loader(ent), F);
    finish(ent, s[(int)(ent & 0xFFFFFFu)], F, x0, acc);
  }

  // integer energy sums G[t] = sum_k wq[k] F[k][t] of the four sites (flip of site t
  // changes the energy by (1 - 2 o_t) G[t] quantised units)
  __device__ __forceinline__ void word_sums(const uint32_t (&F)[NF], int (&G)[4]) const {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      G[t] = 0;
#pragma unroll
      for (int k = 0; k < NF; ++k) G[t] += rule.w->wq[k] * (int)((F[k] >> (8 * t)) & 0xFFu);
    }
  }

  // four decisions from the word's features F and value v, write-back of the flips
  __device__ __forceinline__ void finish(uint32_t ent, uint32_t v, const uint32_t (&F)[NF], const uint32_t (&x0)[4],
                                         int (&acc)[NSLOT]) const {
    int G[4];
    word_sums(F, G);
    finish_g(ent, v, F, G, x0, acc);
  }

  // the same with the integer energy sums given
  __device__ __forceinline__ void finish_g(uint32_t ent, uint32_t v, const uint32_t (&F)[NF], const int (&G)[4],
                                           const uint32_t (&x0)[4], int (&acc)[NSLOT]) const {
    uint32_t sgn;
    const uint32_t flip = decide_store(ent, v, F, G, x0, acc, sgn);
    accumulate(F, flip, sgn, acc);
  }

  // correlation changes of the accepted flips (flip: set bit per accepted site, sgn: its
  // signed change of the site function per byte)
  __device__ __forceinline__ void accumulate(const uint32_t (&F)[NF], uint32_t flip, uint32_t sgn,
                                             int (&acc)[NSLOT]) const {
    if (flip) {
      acc[0] += __popc(flip);
      // sum over the four sites of dpsi * F[k]: signed byte dot product
#pragma unroll
      for (int k = 0; k < NF; ++k) acc[B::feat_class(k)] += __dp4a((int)F[k], (int)sgn, 0);
    }
  }

  // decisions and write-back of the flips; returns the flip mask and sets sgn
  __device__ __forceinline__ uint32_t decide_store(uint32_t ent, uint32_t v, const uint32_t (&F)[NF],
                                                   const int (&G)[4], const uint32_t (&x0)[4], int (&acc)[NSLOT],
                                                   uint32_t& sgn) const {
    const int pw = (int)(ent & 0xFFFFFFu);
    const uint32_t flags = ent >> 24;
    // FP32 decisions of the four sites (branch-free, interleaved)
    bool acc32[4], amb[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int o = (int)((v >> (8 * t)) & 1u);
      acc32[t] = rule.fast(o, 1 - o, o ? -G[t] : G[t], x0[t], amb[t]);
    }
    // exact FP64 decisions where the FP32 one is ambiguous (rare)
    if (amb[0] || amb[1] || amb[2] || amb[3]) {
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (amb[t]) {
          const int o = (int)((v >> (8 * t)) & 1u);
          const int dpsi[1] = {1 - 2 * o};
          acc32[t] = rule.exact(o, 1 - o, dpsi, QuadFeature<NF>{F, 8 * t}, x0[t], acc32[t], acc);
        }
      }
    }
    uint32_t flip = 0u;
    sgn = 0u;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const uint32_t bit = 1u << (8 * t);
      if (acc32[t]) {
        flip |= bit;
        sgn |= (v & bit) ? (0xFFu << (8 * t)) : bit;
      }
    }
    if (flip) {
      const uint32_t nv = v ^ flip;
      uint32_t vi = nv;
      int oi = 0;
      if (flags & 1u) {
        oi = Q;
        vi = __funnelshift_r(nv, nv, 8);
      } else if (flags & 2u) {
        oi = -Q;
        vi = __funnelshift_l(nv, nv, 8);
      }
      const int oj = (flags & 4u) ? dJ : ((flags & 8u) ? -dJ : 0);
      auto put = [&](uint32_t* r) {
        r[0] = nv;
        if (oi) r[oi] = vi;
        if (oj) r[oj] = nv;
        if (oi && oj) r[oi + oj] = vi;
      };
      put(s + pw);
      if (flags & 16u) put(s_prev + pw + dKp);
      if (flags & 32u) put(s_next + pw - dKn);
    }
    return flip;
  }
};

// ---- word layout of the ternary Chebyshev basis
//
// The same four-sites-per-word lattice (bytes hold occupants 0, 1, 2) and row slabs as the
// binary word layout.  A site's local features are linear in byte-parallel monomial counts
// of the indicators u = [o != 1] and s = [o == 2] of its neighbours (B::counts_quad; F[k] =
// tq_const(k) + sum_j tq_coef(k, j) M[j], exact integers), so the four sites' energy sums
// G_b = sum over features of basis b of wq[k] F[k] come from the counts with the weights
// gc[b] + sum_j W[b][j] M[j] (int32, exact modulo 2^32 and equal to the per-site sums).
// Random numbers are those of the per-site (byte) layout: Philox block with counter
// (site, pass, chain, tag) per site, word 0 for the acceptance and bit 31 of word 1 for the
// target occupant; decisions use the same FP32 rule and FP64 re-decision, so trajectories
// equal the byte layout's.
template <int NJ>
struct TernQuadWeights {
  int W[2][NJ];
  int gc[2];
};

// FP64 re-decision of one site of a word (MetropolisRule::exact) with its features from the
// counts: returns bit 0 the decision and bit 1 whether FP32 mode flipped it.  Kept out of
// line: it is taken for few proposals and would otherwise enlarge the update's registers.
template <class B>
__device__ __noinline__ int tern_exact(const MetropolisRule<B>& rule, int o, int o2, int dpsi0, int dpsi1,
                                       const uint32_t* M, int shift, uint32_t x0, bool acc32) {
  struct Fi {
    const uint32_t* M;
    int shift;
    __device__ __forceinline__ int operator()(int k) const {
      int v = B::tq_const(k);
#pragma unroll
      for (int j = 0; j < B::NCOUNT; ++j)
        if (B::tq_coef(k, j) != 0) v += B::tq_coef(k, j) * (int)((M[j] >> shift) & 0xFFu);
      return v;
    }
  };
  int cnt[CeSlots<B::NCLASS>::N] = {};
  const int dpsi[2] = {dpsi0, dpsi1};
  const bool a = rule.exact(o, o2, dpsi, Fi{M, shift}, x0, acc32, cnt);
  return (a ? 1 : 0) | (cnt[B::NCLASS + 1] ? 2 : 0);
}

// GMEM: the window is one chain's lattice in global memory shared by the CTAs of a grid
// sweep (ce_sweep_tgrid_kernel): its words are read with ld.global.cg and written with
// st.global.cg, so no SM keeps a stale copy in L1 across the grid barriers
template <class B, bool GMEM = false>
struct TernQuadSweeper {
  static constexpr int NF = B::NFEAT;
  static constexpr int NC = B::NCLASS;
  static constexpr int NSLOT = CeSlots<NC>::N;
  static constexpr int NJ = B::NCOUNT;
  static_assert(B::NSPECIES == 3 && B::NFUNC == 2, "ternary word layout needs the three-species basis");
  uint32_t* s;
  uint32_t* s_prev;
  uint32_t* s_next;
  int RS, RSY;
  int Q, dJ, dKp, dKn;
  MetropolisRule<B> rule;
  const TernQuadWeights<NJ>* tw;

  __device__ __forceinline__ WordLoaderT<GMEM> loader(uint32_t ent) const {
    return WordLoaderT<GMEM>{s + (int)(ent & 0xFFFFFFu), RS, RSY};
  }

  // one word: counts, the four sites' decisions (Philox block per site), write-back of the
  // accepted changes and their correlation changes
  __device__ __forceinline__ void update(uint32_t ent, uint32_t site0, uint32_t pass, uint32_t chain_id,
                                         uint32_t key0, uint32_t key1, int (&acc)[NSLOT]) const {
    const int pw = (int)(ent & 0xFFFFFFu);
    uint32_t v;
    if constexpr (GMEM)
      v = __ldcg(s + pw);
    else
      v = s[pw];
    uint32_t M[NJ];
    B::counts_quad(loader(ent), M);
    uint32_t nv = v, sg0 = 0u, sg1 = 0u;
    int n_acc = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const U32x4 x = philox4x32_10(U32x4{site0 + (uint32_t)(t * Q), pass, chain_id, SWEEP_TAG}, key0, key1);
      const int o = (int)((v >> (8 * t)) & 0xFFu);
      const int o2 = (o + 1 + (int)(x.y >> 31)) % 3;
      const int dpsi[2] = {B::psi(0, o2) - B::psi(0, o), B::psi(1, o2) - B::psi(1, o)};
      int G0 = tw->gc[0], G1 = tw->gc[1];
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const int m = (int)((M[j] >> (8 * t)) & 0xFFu);
        G0 += tw->W[0][j] * m;
        G1 += tw->W[1][j] * m;
      }
      bool amb;
      bool a = rule.fast(o, o2, dpsi[0] * G0 + dpsi[1] * G1, x.x, amb);
      if (amb) {
        // rare: the FP64 decision out of line, from a copy of the counts
        uint32_t Mc[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) Mc[j] = M[j];
        const int r = tern_exact<B>(rule, o, o2, dpsi[0], dpsi[1], Mc, 8 * t, x.x, a);
        a = (r & 1) != 0;
        acc[NC] += 1;
        acc[NC + 1] += (r >> 1) & 1;
      }
      if (a) {
        nv = (nv & ~(0xFFu << (8 * t))) | ((uint32_t)o2 << (8 * t));
        sg0 |= (uint32_t)(dpsi[0] & 0xFF) << (8 * t);
        sg1 |= (uint32_t)(dpsi[1] & 0xFF) << (8 * t);
        ++n_acc;
      }
    }
    if (n_acc) {
      const uint32_t flags = ent >> 24;
      uint32_t vi = nv;
      int oi = 0;
      if (flags & 1u) {
        oi = Q;
        vi = __funnelshift_r(nv, nv, 8);
      } else if (flags & 2u) {
        oi = -Q;
        vi = __funnelshift_l(nv, nv, 8);
      }
      const int oj = (flags & 4u) ? dJ : ((flags & 8u) ? -dJ : 0);
      auto st = [&](uint32_t* r, uint32_t x) {
        if constexpr (GMEM)
          __stcg(r, x);
        else
          *r = x;
      };
      auto put = [&](uint32_t* r) {
        st(r, nv);
        if (oi) st(r + oi, vi);
        if (oj) st(r + oj, nv);
        if (oi && oj) st(r + oi + oj, vi);
      };
      put(s + pw);
      if (flags & 16u) put(s_prev + pw + dKp);
      if (flags & 32u) put(s_next + pw - dKn);
      // correlation changes: sum over the accepted sites of dpsi_b * F[k] =
      // tq_const(k) sum dpsi_b + sum_j tq_coef(k, j) (signed byte dot product of M[j], dpsi_b)
      acc[0] += n_acc;
      const int c0 = __dp4a((int)0x01010101, (int)sg0, 0), c1 = __dp4a((int)0x01010101, (int)sg1, 0);
#pragma unroll
      for (int k = 0; k < NF; ++k)
        if (B::tq_const(k) != 0) acc[B::feat_class(k)] += B::tq_const(k) * (B::feat_b(k) == 0 ? c0 : c1);
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const int d0 = __dp4a((int)M[j], (int)sg0, 0), d1 = __dp4a((int)M[j], (int)sg1, 0);
#pragma unroll
        for (int k = 0; k < NF; ++k)
          if (B::tq_coef(k, j) != 0) acc[B::feat_class(k)] += B::tq_coef(k, j) * (B::feat_b(k) == 0 ? d0 : d1);
      }
    }
  }
};

template <int NFEAT, int NJ>
struct CeTQuadArgs {
  CeQuadArgs<NFEAT> q;
  TernQuadWeights<NJ> tw;
};

// Word-layout sweep of the ternary basis (one or S CTAs per chain in a cluster, row slabs);
// the structure of ce_sweep_quad_kernel without the pipelined prefetch.
template <class B, int NT>
__global__ void __launch_bounds__(NT, 1)
    ce_sweep_tquad_kernel(const __grid_constant__ CeTQuadArgs<B::NFEAT, B::NCOUNT> TA) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  const CeQuadArgs<B::NFEAT>& A = TA.q;
  extern __shared__ __align__(16) uint32_t sq[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];

  const QuadGeometry& g = A.g;
  const int S = g.S;
  const int chain = blockIdx.x / S;
  int rank = 0;
  cg::cluster_group cluster = cg::this_cluster();
  if (S > 1) rank = (int)cluster.block_rank();
  auto barrier = [&]() {
    if (S > 1)
      cluster.sync();
    else
      __syncthreads();
  };

  const int Q = g.Q, RS = g.RS, RY = g.RY, RSY = RS * RY;
  const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
  const RowSlab sl = row_slab(L1, L2, S, rank, g.planes);
  const int rprev = (rank + S - 1) % S;
  const long long N = (long long)L0 * L1 * L2;
  int8_t* gocc = A.occ + (size_t)chain * N;

  load_word_window<B::HALO>(sq, gocc, L0, L1, L2, Q, RS, RY, sl.kb, sl.nk, threadIdx.x, NT);
  if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;
  const CeChainParams* cpg = A.cp + chain;
  load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
  const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
  const int* cstart = g.color_start + rank * (g.n_colors + 1);

  TernQuadSweeper<B> sw;
  sw.s = sq;
  sw.s_prev = sq;
  sw.s_next = sq;
  if (S > 1) {
    sw.s_prev = cluster.map_shared_rank(sq, (unsigned)rprev);
    sw.s_next = cluster.map_shared_rank(sq, (unsigned)((rank + 1) % S));
  }
  sw.RS = RS;
  sw.RSY = RSY;
  sw.Q = Q;
  sw.dJ = L1 * RS;
  sw.dKp = sl.dkp * RSY;
  sw.dKn = sl.dkn * RSY;
  sw.rule = MetropolisRule<B>{dmu32_sm, dmu64_sm, &A.w, cpg->beta, cpg->beta_log2e, cpg->dtol, cpg->eps,
                              A.precision};
  sw.tw = &TA.tw;
  const int lane = threadIdx.x & 31;
  int acc[NSLOT];
#pragma unroll
  for (int q = 0; q < NSLOT; ++q) acc[q] = 0;
  barrier();

#pragma unroll 1
  for (int pass = 0; pass < A.n_passes; ++pass) {
    const uint32_t pass_g = (uint32_t)(A.pass0 + pass);
#pragma unroll 1
    for (int c = 0; c < g.n_colors; ++c) {
#pragma unroll 1
      for (int e = cstart[c] + threadIdx.x; e < cstart[c + 1]; e += NT)
        sw.update(__ldg(g.entries + e), __ldg(g.site_l + e), pass_g, chain_id, key0, key1, acc);
      barrier();
      if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
        int* buf = acc_sm[(pass - 1) & 1];
        const int v = buf[threadIdx.x];
        buf[threadIdx.x] = 0;
        if (v)
          atomicAdd(reinterpret_cast<unsigned long long*>(
                        A.out + ((size_t)(pass - 1) * A.n_chains + chain) * NSLOT + threadIdx.x),
                    (unsigned long long)(long long)v);
      }
    }
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) {
      const int v = warp_sum(acc[q]);
      if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
      acc[q] = 0;
    }
  }
  barrier();
  if (A.n_passes > 0 && threadIdx.x < NSLOT) {
    const int pl = A.n_passes - 1;
    int* buf = acc_sm[pl & 1];
    const int v = buf[threadIdx.x];
    if (v)
      atomicAdd(reinterpret_cast<unsigned long long*>(A.out + ((size_t)pl * A.n_chains + chain) * NSLOT + threadIdx.x),
                (unsigned long long)(long long)v);
  }
  store_word_rows<B::HALO>(sq, gocc, L0, L1, Q, RS, RY, sl, threadIdx.x, NT);
  barrier();
}

// Barrier of the CTAs of one chain in a cooperative launch (every CTA resident): one
// arrival counter and one generation word per chain in global memory; the last CTA to
// arrive resets the counter and advances the generation.  Waits are bounded: a CTA that
// polls kGridSpinLimit times without the generation moving records status 3 and sets the
// abort word, and every waiting CTA leaves at its next poll; the kernel then returns
// without writing the occupations back.
constexpr unsigned kGridSpinLimit = 1u << 22;  // polls of >= 64 ns each: well over a second

struct GridBarrier {
  unsigned* count;  // [n_chains]
  unsigned* gen;    // [n_chains]
  int* status;      // 0, or 3: a barrier wait ran out
  int* abort;       // non-zero: leave the sweep
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// all CTAs of `chain` (n_ctas of them) reach this point; returns false after an abort
__device__ __forceinline__ bool grid_chain_sync(const GridBarrier& gb, int chain, unsigned n_ctas, int* s_flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int stop = 0;
    const unsigned g0 = ld_acquire_gpu(gb.gen + chain);
    __threadfence();
    if (atomicAdd(gb.count + chain, 1u) + 1u == n_ctas) {
      atomicExch(gb.count + chain, 0u);
      __threadfence();
      atomicAdd(gb.gen + chain, 1u);
    } else {
      unsigned polls = 0;
      while (ld_acquire_gpu(gb.gen + chain) == g0) {
        if (*(volatile int*)gb.abort) {
          stop = 1;
          break;
        }
        if (++polls > kGridSpinLimit) {
          atomicExch(gb.status, 3);
          atomicExch(gb.abort, 1);
          stop = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    *s_flag = stop | *(volatile int*)gb.abort;
  }
  __syncthreads();
  return *s_flag == 0;
}

template <int NFEAT, int NJ>
struct CeTGridArgs {
  CeTQuadArgs<NFEAT, NJ> t;  // geometry of the one-slab (S = 1) word window and lists
  uint32_t* win;             // [n_chains][win_words] the chains' windows in global memory
  long long win_words;
  int G;                     // CTAs per chain
  GridBarrier gb;
};

// Grid sweep of the ternary word layout for chains too large for one cluster to sweep
// quickly (a single 96^3 chain holds 16 of 152 SMs in a 16-CTA cluster): each chain's whole
// padded window (the S = 1 window of ce_sweep_tquad_kernel) lives in global memory and L2,
// G CTAs share each colour's word list (word e of the colour to thread e mod G*NT), and a
// grid barrier per chain separates the colours.  Same words, neighbours, random numbers and
// decisions as the cluster kernels, so the trajectories are identical.
template <class B, int NT>
__global__ void __launch_bounds__(NT, 1)
    ce_sweep_tgrid_kernel(const __grid_constant__ CeTGridArgs<B::NFEAT, B::NCOUNT> GA) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  const CeQuadArgs<B::NFEAT>& A = GA.t.q;
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];
  __shared__ int s_flag;

  const QuadGeometry& g = A.g;
  const int G = GA.G;
  const int chain = blockIdx.x / G, part = blockIdx.x % G;
  const int Q = g.Q, RS = g.RS, RY = g.RY, RSY = RS * RY;
  const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
  const long long N = (long long)L0 * L1 * L2;
  int8_t* gocc = A.occ + (size_t)chain * N;
  uint32_t* win = GA.win + (size_t)chain * GA.win_words;
  const int gtid = part * NT + threadIdx.x, gthreads = G * NT;

  load_word_window<B::HALO>(win, gocc, L0, L1, L2, Q, RS, RY, 0, L2, gtid, gthreads);
  if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;
  const CeChainParams* cpg = A.cp + chain;
  load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
  const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
  const int* cstart = g.color_start;

  TernQuadSweeper<B, true> sw;
  sw.s = win;
  sw.s_prev = win;
  sw.s_next = win;
  sw.RS = RS;
  sw.RSY = RSY;
  sw.Q = Q;
  sw.dJ = L1 * RS;
  sw.dKp = L2 * RSY;  // the one slab's halo images: L2 planes up and down
  sw.dKn = L2 * RSY;
  sw.rule = MetropolisRule<B>{dmu32_sm, dmu64_sm, &A.w, cpg->beta, cpg->beta_log2e, cpg->dtol, cpg->eps,
                              A.precision};
  sw.tw = &GA.t.tw;
  const int lane = threadIdx.x & 31;
  int acc[NSLOT];
#pragma unroll
  for (int q = 0; q < NSLOT; ++q) acc[q] = 0;
  bool ok = grid_chain_sync(GA.gb, chain, (unsigned)G, &s_flag);

#pragma unroll 1
  for (int pass = 0; ok && pass < A.n_passes; ++pass) {
    const uint32_t pass_g = (uint32_t)(A.pass0 + pass);
#pragma unroll 1
    for (int c = 0; c < g.n_colors; ++c) {
#pragma unroll 1
      for (int e = cstart[c] + gtid; e < cstart[c + 1]; e += gthreads)
        sw.update(__ldg(g.entries + e), __ldg(g.site_l + e), pass_g, chain_id, key0, key1, acc);
      ok = grid_chain_sync(GA.gb, chain, (unsigned)G, &s_flag);
      if (!ok) break;
      if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
        int* buf = acc_sm[(pass - 1) & 1];
        const int v = buf[threadIdx.x];
        buf[threadIdx.x] = 0;
        if (v)
          atomicAdd(reinterpret_cast<unsigned long long*>(
                        A.out + ((size_t)(pass - 1) * A.n_chains + chain) * NSLOT + threadIdx.x),
                    (unsigned long long)(long long)v);
      }
    }
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) {
      const int v = warp_sum(acc[q]);
      if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
      acc[q] = 0;
    }
  }
  if (!ok) return;
  __syncthreads();
  if (A.n_passes > 0 && threadIdx.x < NSLOT) {
    const int pl = A.n_passes - 1;
    const int v = acc_sm[pl & 1][threadIdx.x];
    if (v)
      atomicAdd(reinterpret_cast<unsigned long long*>(A.out + ((size_t)pl * A.n_chains + chain) * NSLOT + threadIdx.x),
                (unsigned long long)(long long)v);
  }
  // the owned rows back to the occupation array (words read past L1: other SMs wrote them)
  for (long long idx = gtid; idx < (long long)Q * L1 * L2; idx += gthreads) {
    const int w = (int)(idx % Q);
    const long long R = idx / Q;
    const int j = (int)(R % L1), k = (int)(R / L1);
    const uint32_t word = __ldcg(win + (w + B::HALO) + (size_t)RS * ((j + B::HALO) + (size_t)RY * (k + B::HALO)));
    int8_t* row = gocc + (long long)L0 * (j + (long long)L1 * k);
#pragma unroll
    for (int t = 0; t < 4; ++t) row[w + t * Q] = (int8_t)((word >> (8 * t)) & 0xFFu);
  }
}

// Philox block of the first word of a thread in one colour phase: its four sites take
// words 0..3 of the block with counter (site of byte 0, pass, chain, tag)
struct QuadPrefetch {
  uint32_t ent, x0[4];

  template <int NT>
  __device__ __forceinline__ void prepare(const int* cstart, int c, const uint32_t* entries,
                                          const uint32_t* site_l, int Q, uint32_t pass, uint32_t chain_id,
                                          uint32_t key0, uint32_t key1) {
    const int e = cstart[c] + threadIdx.x;
    if (e < cstart[c + 1]) {
      ent = __ldg(entries + e);
      const U32x4 x = philox4x32_10(U32x4{__ldg(site_l + e), pass, chain_id, SWEEP_TAG}, key0, key1);
      x0[0] = x.x;
      x0[1] = x.y;
      x0[2] = x.z;
      x0[3] = x.w;
    }
  }
};

// Pipelined variant (colouring with a generated early/late split, B::Pipe<P>): besides
// the Philox block, the first word's early() part (every neighbour not of the colour
// proposed just before) is computed between the cluster arrive and wait of the previous
// phase; after the wait only late() remains.
template <class B, int P>
struct QuadPipePrefetch {
  uint32_t ent, x0[4];
  typename B::template Pipe<P>::State st;

  template <int NT>
  __device__ __forceinline__ void prepare(const QuadSweeper<B>& sw, const int* cstart, int c, const uint32_t* entries,
                                          const uint32_t* site_l, uint32_t pass, uint32_t chain_id, uint32_t key0,
                                          uint32_t key1) {
    const int e = cstart[c] + threadIdx.x;
    if (e < cstart[c + 1]) {
      ent = __ldg(entries + e);
      const U32x4 x = philox4x32_10(U32x4{__ldg(site_l + e), pass, chain_id, SWEEP_TAG}, key0, key1);
      x0[0] = x.x;
      x0[1] = x.y;
      x0[2] = x.z;
      x0[3] = x.w;
      B::template Pipe<P>::early(sw.loader(ent), st);
    }
  }
};

template <class B, int NT, int P>
__device__ __forceinline__ void sweep_phase_quad_pipe(const QuadSweeper<B>& sw, const QuadPipePrefetch<B, P>& pf,
                                                      const int* cstart, int c, const uint32_t* entries,
                                                      const uint32_t* site_l, uint32_t pass, uint32_t chain_id,
                                                      uint32_t key0, uint32_t key1,
                                                      int (&acc)[QuadSweeper<B>::NSLOT]) {
  const int e0 = cstart[c] + threadIdx.x, e_end = cstart[c + 1];
  if (e0 < e_end) {
    uint32_t F[B::NFEAT], Lw[B::template Pipe<P>::NGROUP];
    B::template Pipe<P>::late(sw.loader(pf.ent), pf.st, F, Lw);
    sw.finish(pf.ent, pf.st.own, F, pf.x0, acc);
  }
#pragma unroll 1
  for (int e = e0 + NT; e < e_end; e += NT) {
    const uint32_t ent = __ldg(entries + e);
    const U32x4 x = philox4x32_10(U32x4{__ldg(site_l + e), pass, chain_id, SWEEP_TAG}, key0, key1);
    const uint32_t x0[4] = {x.x, x.y, x.z, x.w};
    sw.update(ent, x0, acc);
  }
}

template <class B, int NT>
__device__ __forceinline__ void sweep_phase_quad(const QuadSweeper<B>& sw, const QuadPrefetch& pf, const int* cstart,
                                                 int c, const uint32_t* entries, const uint32_t* site_l,
                                                 uint32_t pass, uint32_t chain_id, uint32_t key0, uint32_t key1,
                                                 int (&acc)[QuadSweeper<B>::NSLOT]) {
  const int e0 = cstart[c] + threadIdx.x, e_end = cstart[c + 1];
  if (e0 < e_end) sw.update(pf.ent, pf.x0, acc);
#pragma unroll 1
  for (int e = e0 + NT; e < e_end; e += NT) {
    const uint32_t ent = __ldg(entries + e);
    const U32x4 x = philox4x32_10(U32x4{__ldg(site_l + e), pass, chain_id, SWEEP_TAG}, key0, key1);
    const uint32_t x0[4] = {x.x, x.y, x.z, x.w};
    sw.update(ent, x0, acc);
  }
}

// PIPE < 0: generic word layout; PIPE >= 0: pipelined features for colouring B::Pipe<PIPE>
template <class B, int NT, int PIPE>
__global__ void __launch_bounds__(NT, 1) ce_sweep_quad_kernel(const __grid_constant__ CeQuadArgs<B::NFEAT> A) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  extern __shared__ __align__(16) uint32_t sq[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];

  const QuadGeometry& g = A.g;
  const int S = g.S;
  const int chain = blockIdx.x / S;
  int rank = 0;
  cg::cluster_group cluster = cg::this_cluster();
  if (S > 1) rank = (int)cluster.block_rank();
  auto barrier = [&]() {
    if (S > 1)
      cluster.sync();
    else
      __syncthreads();
  };

  const int Q = g.Q, RS = g.RS, RY = g.RY, RSY = RS * RY;
  const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
  const RowSlab sl = row_slab(L1, L2, S, rank, g.planes);
  const int rprev = (rank + S - 1) % S;
  const long long N = (long long)L0 * L1 * L2;
  int8_t* gocc = A.occ + (size_t)chain * N;

  // ---- load the slab's window
  load_word_window<B::HALO>(sq, gocc, L0, L1, L2, Q, RS, RY, sl.kb, sl.nk, threadIdx.x, NT);
  if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;

  const CeChainParams* cpg = A.cp + chain;
  load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
  const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
  const int* cstart = g.color_start + rank * (g.n_colors + 1);

  QuadSweeper<B> sw;
  sw.s = sq;
  sw.s_prev = sq;
  sw.s_next = sq;
  if (S > 1) {
    sw.s_prev = cluster.map_shared_rank(sq, (unsigned)rprev);
    sw.s_next = cluster.map_shared_rank(sq, (unsigned)((rank + 1) % S));
  }
  sw.RS = RS;
  sw.RSY = RSY;
  sw.Q = Q;
  sw.dJ = L1 * RS;
  sw.dKp = sl.dkp * RSY;
  sw.dKn = sl.dkn * RSY;
  sw.rule = MetropolisRule<B>{dmu32_sm, dmu64_sm, &A.w, cpg->beta, cpg->beta_log2e, cpg->dtol, cpg->eps,
                              A.precision};
  const int lane = threadIdx.x & 31;
  int acc[NSLOT];
#pragma unroll
  for (int q = 0; q < NSLOT; ++q) acc[q] = 0;

  using Prefetch =
      typename std::conditional<(PIPE >= 0), QuadPipePrefetch<B, (PIPE >= 0 ? PIPE : 0)>, QuadPrefetch>::type;
  Prefetch pf;
  auto prepare = [&](int c, uint32_t pass) {
    if constexpr (PIPE >= 0)
      pf.template prepare<NT>(sw, cstart, c, g.entries, g.site_l, pass, chain_id, key0, key1);
    else
      pf.template prepare<NT>(cstart, c, g.entries, g.site_l, Q, pass, chain_id, key0, key1);
  };
  barrier();
  prepare(0, (uint32_t)A.pass0);  // the pipelined prefetch reads the loaded slab

#pragma unroll 1
  for (int pass = 0; pass < A.n_passes; ++pass) {
    const uint32_t pass_g = (uint32_t)(A.pass0 + pass);
#pragma unroll 1
    for (int c = 0; c < g.n_colors; ++c) {
      if constexpr (PIPE >= 0)
        sweep_phase_quad_pipe<B, NT, (PIPE >= 0 ? PIPE : 0)>(sw, pf, cstart, c, g.entries, g.site_l, pass_g,
                                                             chain_id, key0, key1, acc);
      else
        sweep_phase_quad<B, NT>(sw, pf, cstart, c, g.entries, g.site_l, pass_g, chain_id, key0, key1, acc);
      const bool last = (c + 1 == g.n_colors);
      // arrive, prepare the next phase (Philox block; pipelined: the early features,
      // which read no word of colour c) while other threads finish, then wait
      if (S > 1) {
        cluster_arrive_release();
        prepare(last ? 0 : c + 1, last ? pass_g + 1 : pass_g);
        cluster_wait_acquire();
      } else {
        __syncthreads();
        prepare(last ? 0 : c + 1, last ? pass_g + 1 : pass_g);
      }
      if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
        int* buf = acc_sm[(pass - 1) & 1];
        const int v = buf[threadIdx.x];
        buf[threadIdx.x] = 0;
        if (v)
          atomicAdd(reinterpret_cast<unsigned long long*>(
                        A.out + ((size_t)(pass - 1) * A.n_chains + chain) * NSLOT + threadIdx.x),
                    (unsigned long long)(long long)v);
      }
    }
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) {
      const int v = warp_sum(acc[q]);
      if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
      acc[q] = 0;
    }
  }
  barrier();
  if (A.n_passes > 0 && threadIdx.x < NSLOT) {
    const int pl = A.n_passes - 1;
    int* buf = acc_sm[pl & 1];
    const int v = buf[threadIdx.x];
    if (v)
      atomicAdd(reinterpret_cast<unsigned long long*>(A.out + ((size_t)pl * A.n_chains + chain) * NSLOT + threadIdx.x),
                (unsigned long long)(long long)v);
  }
  // ---- write back own words
  store_word_rows<B::HALO>(sq, gocc, L0, L1, Q, RS, RY, sl, threadIdx.x, NT);
  barrier();
}

// ---- warp-specialised pipelined word sweep
//
// Two roles of NW threads each share a CTA.  During colour phase g the finish role takes
// the decisions of phase g's words (late features, four FP32/FP64 decisions, write-back,
// correlation changes) while the early role prepares phase g+1's words (Philox block,
// early feature and energy sums, which read no word of colour g) into a double-buffered
// staging area
// in shared memory.  Both roles meet at the phase's cluster barrier, so a phase costs about
// the longer of the two roles rather than their sum.  Requires at most NW words per
// (CTA, colour) and a generated pipeline colouring; trajectories equal the other kernels'.
template <class B, int P>
struct WsStage {
  using State = typename B::template Pipe<P>::State;
  static constexpr int NF = B::NFEAT;
  static constexpr int NK = B::template Pipe<P>::NKEEP;
  static constexpr int NG = B::template Pipe<P>::NGROUP;
  // E, K, own, entry, Philox words x0[4], early energy sums GE[4], late-group coefficients A[NG][4]
  static constexpr int NFIELD = NF + NK + 2 + 4 + 4 + 4 * NG;

  // the early part of the integer energy sums and, per late group g, the amount it adds
  // to a site's sum when set: GE[t] = sum_k wq[k] E[k][t], A[g][t] = sum over the group's
  // terms (feature k, kept word K or none, count n) of wq[k] n (K[t] or 1)
  __device__ __forceinline__ static void sums(const State& st, const int* wq, int (&GE)[4], int (&A)[NG][4]) {
    using PP = typename B::template Pipe<P>;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      GE[t] = 0;
#pragma unroll
      for (int k = 0; k < NF; ++k) GE[t] += wq[k] * (int)((st.E[k] >> (8 * t)) & 0xFFu);
#pragma unroll
      for (int g = 0; g < NG; ++g) A[g][t] = 0;
#pragma unroll
      for (int i = 0; i < PP::NTERM; ++i) {
        const int kk = PP::term_keep(i);
        const int val = kk < 0 ? 1 : (int)((st.K[kk < 0 ? 0 : kk] >> (8 * t)) & 0xFFu);
        A[PP::term_group(i)][t] += wq[PP::term_feature(i)] * PP::term_count(i) * val;
      }
    }
  }

  // field-major: base[field * NW + word]
  template <int NW>
  __device__ __forceinline__ static void store(uint32_t* base, int w, const State& st, uint32_t ent,
                                               const uint32_t (&x0)[4], const int (&GE)[4], const int (&A)[NG][4]) {
#pragma unroll
    for (int k = 0; k < NF; ++k) base[k * NW + w] = st.E[k];
#pragma unroll
    for (int k = 0; k < NK; ++k) base[(NF + k) * NW + w] = st.K[k];
    base[(NF + NK) * NW + w] = st.own;
    base[(NF + NK + 1) * NW + w] = ent;
#pragma unroll
    for (int t = 0; t < 4; ++t) base[(NF + NK + 2 + t) * NW + w] = x0[t];
#pragma unroll
    for (int t = 0; t < 4; ++t) base[(NF + NK + 6 + t) * NW + w] = (uint32_t)GE[t];
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
      for (int t = 0; t < 4; ++t) base[(NF + NK + 10 + 4 * g + t) * NW + w] = (uint32_t)A[g][t];
  }
  template <int NW>
  __device__ __forceinline__ static void load(const uint32_t* base, int w, State& st, uint32_t& ent,
                                              uint32_t (&x0)[4], int (&GE)[4], int (&A)[NG][4]) {
#pragma unroll
    for (int k = 0; k < NF; ++k) st.E[k] = base[k * NW + w];
#pragma unroll
    for (int k = 0; k < NK; ++k) st.K[k] = base[(NF + k) * NW + w];
    st.own = base[(NF + NK) * NW + w];
    ent = base[(NF + NK + 1) * NW + w];
#pragma unroll
    for (int t = 0; t < 4; ++t) x0[t] = base[(NF + NK + 2 + t) * NW + w];
#pragma unroll
    for (int t = 0; t < 4; ++t) GE[t] = (int)base[(NF + NK + 6 + t) * NW + w];
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
      for (int t = 0; t < 4; ++t) A[g][t] = (int)base[(NF + NK + 10 + 4 * g + t) * NW + w];
  }
};

template <class B, int NW, int PIPE>
__global__ void __launch_bounds__(2 * NW, 1) ce_sweep_ws_kernel(const __grid_constant__ CeQuadArgs<B::NFEAT> A) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  using Stage = WsStage<B, PIPE>;
  using State = typename Stage::State;
  extern __shared__ __align__(16) uint32_t sq[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];

  const QuadGeometry& g = A.g;
  const int S = g.S;
  const int slot_i = blockIdx.x / S;
  const int chain = A.n_map > 0 ? A.map_chain[slot_i] : slot_i;
  const long long pbase = A.n_map > 0 ? (long long)A.map_pass[slot_i] : 0ll;  // output row of pass 0
  const long long pass0 = A.pass0 + pbase;
  int rank = 0;
  cg::cluster_group cluster = cg::this_cluster();
  if (S > 1) rank = (int)cluster.block_rank();
  auto barrier = [&]() {
    if (S > 1)
      cluster.sync();
    else
      __syncthreads();
  };
  const bool finisher = threadIdx.x < NW;
  const int tid = finisher ? threadIdx.x : threadIdx.x - NW;

  const int Q = g.Q, RS = g.RS, RY = g.RY, RSY = RS * RY;
  const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
  const RowSlab sl = row_slab(L1, L2, S, rank, g.planes);
  const int rprev = (rank + S - 1) % S;
  const long long N = (long long)L0 * L1 * L2;
  int8_t* gocc = A.occ + (size_t)chain * N;
  const int lattice_words = RSY * g.window_planes;
  uint32_t* stage = sq + ((lattice_words + 3) & ~3);  // [2][NFIELD][NW]
  // the CTA's site lists (entries, Philox counter words) and colour starts, copied once
  const int max_words = Q * g.max_rows;
  uint32_t* ents = stage + 2 * Stage::NFIELD * NW;
  uint32_t* sites = ents + max_words;
  int* cst = reinterpret_cast<int*>(sites + max_words);

  // ---- load the slab's window
  load_word_window<B::HALO>(sq, gocc, L0, L1, L2, Q, RS, RY, sl.kb, sl.nk, threadIdx.x, 2 * NW);
  if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;

  const CeChainParams* cpg = A.cp + chain;
  load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
  const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
  {
    const int* cg0 = g.color_start + rank * (g.n_colors + 1);
    const int base = cg0[0], n = cg0[g.n_colors] - base;
    for (int i = threadIdx.x; i <= g.n_colors; i += 2 * NW) cst[i] = cg0[i] - base;
    constexpr int UL = 4;  // loads of UL entries in flight per thread
    for (int i0 = threadIdx.x; i0 < n; i0 += UL * 2 * NW) {
      uint32_t e[UL], t[UL];
#pragma unroll
      for (int u = 0; u < UL; ++u) {
        const int i = i0 + u * 2 * NW;
        if (i < n) {
          e[u] = __ldg(g.entries + base + i);
          t[u] = __ldg(g.site_l + base + i);
        }
      }
#pragma unroll
      for (int u = 0; u < UL; ++u) {
        const int i = i0 + u * 2 * NW;
        if (i < n) {
          ents[i] = e[u];
          sites[i] = t[u];
        }
      }
    }
  }
  const int* cstart = cst;

  QuadSweeper<B> sw;
  sw.s = sq;
  sw.s_prev = sq;
  sw.s_next = sq;
  if (S > 1) {
    sw.s_prev = cluster.map_shared_rank(sq, (unsigned)rprev);
    sw.s_next = cluster.map_shared_rank(sq, (unsigned)((rank + 1) % S));
  }
  sw.RS = RS;
  sw.RSY = RSY;
  sw.Q = Q;
  sw.dJ = L1 * RS;
  sw.dKp = sl.dkp * RSY;
  sw.dKn = sl.dkn * RSY;
  sw.rule = MetropolisRule<B>{dmu32_sm, dmu64_sm, &A.w, cpg->beta, cpg->beta_log2e, cpg->dtol, cpg->eps,
                              A.precision};
  const int lane = threadIdx.x & 31;
  int acc[NSLOT];
#pragma unroll
  for (int q = 0; q < NSLOT; ++q) acc[q] = 0;

  // early role: Philox block, early features and energy sums of word tid of colour c
  // (pass `pass`) into a stage slot
  auto prepare = [&](int c, uint32_t pass, uint32_t* slot) {
    const int e = cstart[c] + tid;
    if (e < cstart[c + 1]) {
      const uint32_t ent = ents[e];
      const U32x4 x = philox4x32_10(U32x4{sites[e], pass, chain_id, SWEEP_TAG}, key0, key1);
      const uint32_t x0[4] = {x.x, x.y, x.z, x.w};
      State st;
      B::template Pipe<PIPE>::early(sw.loader(ent), st);
      int GE[4], Ac[Stage::NG][4];
      Stage::sums(st, A.w.wq, GE, Ac);
      Stage::template store<NW>(slot, tid, st, ent, x0, GE, Ac);
    }
  };
  constexpr int SLOT = Stage::NFIELD * NW;

  barrier();  // slab loaded
  if (!finisher) prepare(0, (uint32_t)pass0, stage);
  barrier();  // stage 0 ready

  int parity = 0;
#pragma unroll 1
  for (int pass = 0; pass < A.n_passes; ++pass) {
    const uint32_t pass_g = (uint32_t)(pass0 + pass);
#pragma unroll 1
    for (int c = 0; c < g.n_colors; ++c) {
      const bool last = (c + 1 == g.n_colors);
      // finish role: decisions and write-back before the arrive; the correlation changes
      // (needed only at the end of the pass) while the barrier completes
      uint32_t F[B::NFEAT], flip = 0u, sgn = 0u;
      if (finisher) {
        if (cstart[c] + tid < cstart[c + 1]) {
          State st;
          uint32_t ent, x0[4];
          int G[4], Ac[Stage::NG][4];
          Stage::template load<NW>(stage + parity * SLOT, tid, st, ent, x0, G, Ac);
          uint32_t Lw[Stage::NG];
          B::template Pipe<PIPE>::late(sw.loader(ent), st, F, Lw);
#pragma unroll
          for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int gi = 0; gi < Stage::NG; ++gi) G[t] += (int)((Lw[gi] >> (8 * t)) & 1u) * Ac[gi][t];
          flip = sw.decide_store(ent, st.own, F, G, x0, acc, sgn);
        }
      } else {
        prepare(last ? 0 : c + 1, last ? pass_g + 1 : pass_g, stage + (parity ^ 1) * SLOT);
      }
      if (S > 1) {
        cluster_arrive_release();
        if (finisher) sw.accumulate(F, flip, sgn, acc);
        cluster_wait_acquire();
      } else {
        if (finisher) sw.accumulate(F, flip, sgn, acc);
        __syncthreads();
      }
      parity ^= 1;
      if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
        int* buf = acc_sm[(pass - 1) & 1];
        const int v = buf[threadIdx.x];
        buf[threadIdx.x] = 0;
        if (v)
          atomicAdd(reinterpret_cast<unsigned long long*>(
                        A.out + ((size_t)(pbase + pass - 1) * A.n_chains + chain) * NSLOT + threadIdx.x),
                    (unsigned long long)(long long)v);
      }
    }
    if (finisher) {
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) {
        const int v = warp_sum(acc[q]);
        if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
        acc[q] = 0;
      }
    }
  }
  barrier();
  if (A.n_passes > 0 && threadIdx.x < NSLOT) {
    const int pl = A.n_passes - 1;
    int* buf = acc_sm[pl & 1];
    const int v = buf[threadIdx.x];
    if (v)
      atomicAdd(reinterpret_cast<unsigned long long*>(A.out + ((size_t)(pbase + pl) * A.n_chains + chain) * NSLOT +
                                                      threadIdx.x),
                (unsigned long long)(long long)v);
  }
  store_word_rows<B::HALO>(sq, gocc, L0, L1, Q, RS, RY, sl, threadIdx.x, 2 * NW);
  barrier();
}

// ---- persistent pool kernel: many chains of any shape, one CTA per chain

// geometry of one supercell shape swept by S CTAs: colour lists per slab
struct PoolGeometry {
  int L0, L1, L2;
  int n_colors;
  int planes;  // word layout: slab kind (row_slab)
  const int* color_start;   // [S][n_colors + 1]
  const uint32_t* entries;  // padded index | flags << 24
  const uint32_t* site_l;
};

// one work item: a chain of some geometry
struct PoolItem {
  int geom;
  int param;             // index into the chain-parameter array
  long long occ_offset;  // into the occupation arena
  long long out_offset;  // into the output array, [pass][NSLOT] for this item
  long long pass0;       // the chain's pass count before this launch (Philox counter)
};

template <int NFEAT>
struct CePoolArgs {
  const PoolGeometry* geoms;
  const PoolItem* items;
  int n_items;
  int* next_item;  // work counter (zeroed by the host)
  CeWeights<NFEAT> w;
  const CeChainParams* cp;
  int8_t* occ;  // arena
  int n_passes;
  int precision;
  long long* out;
};

template <class B, int NT>
__global__ void __launch_bounds__(NT, 1) ce_pool_kernel(const __grid_constant__ CePoolArgs<B::NFEAT> A) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  constexpr int PRE = (NS == 2) ? 3 : 1;
  extern __shared__ __align__(16) int8_t s[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];
  __shared__ int item_sm;
  const int lane = threadIdx.x & 31;

#pragma unroll 1
  while (true) {
    if (threadIdx.x == 0) item_sm = atomicAdd(A.next_item, 1);
    __syncthreads();
    const int it = item_sm;
    if (it >= A.n_items) break;
    const PoolItem item = A.items[it];
    const PoolGeometry g = A.geoms[item.geom];
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int PX = L0 + 2 * B::HALO, PY = L1 + 2 * B::HALO, PXY = PX * PY;
    int8_t* gocc = A.occ + item.occ_offset;
    for (int idx = threadIdx.x; idx < PXY * (L2 + 2 * B::HALO); idx += NT) {
      const int ip = idx % PX, jp = (idx / PX) % PY, kp = idx / PXY;
      int i = ip - B::HALO, j = jp - B::HALO, k = kp - B::HALO;
      i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
      j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
      k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
      s[idx] = B::code_of_occ(gocc[i + (long long)L0 * (j + (long long)L1 * k)]);
    }
    if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;
    const CeChainParams* cpg = A.cp + item.param;
    load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
    const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
    SiteSweeper<B> sw;
    sw.s = s;
    sw.s_prev = s;
    sw.s_next = s;
    sw.PX = PX;
    sw.PXY = PXY;
    sw.dI = L0;
    sw.dJ = L1 * PX;
    sw.dKp = L2 * PXY;
    sw.dKn = L2 * PXY;
    sw.dmu32 = dmu32_sm;
    sw.dmu64 = dmu64_sm;
    sw.w = &A.w;
    sw.beta = cpg->beta;
    sw.beta_log2e = cpg->beta_log2e;
    sw.dtol = cpg->dtol;
    sw.eps = cpg->eps;
    sw.precision = A.precision;
    int acc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) acc[q] = 0;
    long long* out = A.out + item.out_offset;
    PhasePrefetch<PRE> pf;
    pf.template prepare<NT>(g.color_start, 0, g.entries, g.site_l, (uint32_t)item.pass0, chain_id, key0, key1);
    __syncthreads();
#pragma unroll 1
    for (int pass = 0; pass < A.n_passes; ++pass) {
      const uint32_t pass_g = (uint32_t)(item.pass0 + pass);
#pragma unroll 1
      for (int c = 0; c < g.n_colors; ++c) {
        sweep_phase<B, NT, PRE>(sw, pf, g.color_start, c, g.entries, g.site_l, pass_g, chain_id, key0, key1, acc);
        const bool last = (c + 1 == g.n_colors);
        pf.template prepare<NT>(g.color_start, last ? 0 : c + 1, g.entries, g.site_l,
                                last ? pass_g + 1 : pass_g, chain_id, key0, key1);
        __syncthreads();
        if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
          int* buf = acc_sm[(pass - 1) & 1];
          out[(size_t)(pass - 1) * NSLOT + threadIdx.x] = buf[threadIdx.x];
          buf[threadIdx.x] = 0;
        }
      }
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) {
        const int v = warp_sum(acc[q]);
        if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
        acc[q] = 0;
      }
    }
    __syncthreads();
    if (A.n_passes > 0 && threadIdx.x < NSLOT) {
      const int pl = A.n_passes - 1;
      out[(size_t)pl * NSLOT + threadIdx.x] = acc_sm[pl & 1][threadIdx.x];
    }
    for (int idx = threadIdx.x; idx < L0 * L1 * L2; idx += NT) {
      const int i = idx % L0, j = (idx / L0) % L1, k = idx / (L0 * L1);
      const int pidx = (i + B::HALO) + PX * ((j + B::HALO) + PY * (k + B::HALO));
      gocc[i + (long long)L0 * (j + (long long)L1 * k)] = (int8_t)B::occ_of_code(s[pidx]);
    }
    __syncthreads();
  }
}

// Persistent pool kernel for small byte-layout chains, one warp per chain: every warp of
// the CTA takes chains from the work queue on its own and sweeps each in its own window of
// win_bytes bytes of shared memory (padded lattice, periodic borders), the lanes sharing a
// colour's sites and __syncwarp between colours.  A chain of 8^3 sites has 32 sites per
// colour: a CTA per chain would leave all but one warp idle behind CTA barriers.  The site
// update and the per-pass outputs are those of ce_pool_kernel.
template <class B, int NW>
__global__ void __launch_bounds__(32 * NW, 1)
    ce_pool_warp_kernel(const __grid_constant__ CePoolArgs<B::NFEAT> A, int win_bytes) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  extern __shared__ __align__(16) int8_t s_all[];
  __shared__ float dmu32_sm[NW][NS * NS];
  __shared__ double dmu64_sm[NW][NS * NS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t* s = s_all + (size_t)warp * win_bytes;

#pragma unroll 1
  while (true) {
    int it = 0;
    if (lane == 0) it = atomicAdd(A.next_item, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= A.n_items) break;
    const PoolItem item = A.items[it];
    const PoolGeometry g = A.geoms[item.geom];
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int PX = L0 + 2 * B::HALO, PY = L1 + 2 * B::HALO, PXY = PX * PY;
    int8_t* gocc = A.occ + item.occ_offset;
    for (int idx = lane; idx < PXY * (L2 + 2 * B::HALO); idx += 32) {
      const int ip = idx % PX, jp = (idx / PX) % PY, kp = idx / PXY;
      int i = ip - B::HALO, j = jp - B::HALO, k = kp - B::HALO;
      i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
      j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
      k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
      s[idx] = B::code_of_occ(gocc[i + (long long)L0 * (j + (long long)L1 * k)]);
    }
    const CeChainParams* cpg = A.cp + item.param;
    if (lane < NS * NS) {
      dmu32_sm[warp][lane] = cpg->dmu32[lane];
      dmu64_sm[warp][lane] = cpg->dmu64[lane];
    }
    const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
    SiteSweeper<B> sw;
    sw.s = s;
    sw.s_prev = s;
    sw.s_next = s;
    sw.PX = PX;
    sw.PXY = PXY;
    sw.dI = L0;
    sw.dJ = L1 * PX;
    sw.dKp = L2 * PXY;
    sw.dKn = L2 * PXY;
    sw.dmu32 = dmu32_sm[warp];
    sw.dmu64 = dmu64_sm[warp];
    sw.w = &A.w;
    sw.beta = cpg->beta;
    sw.beta_log2e = cpg->beta_log2e;
    sw.dtol = cpg->dtol;
    sw.eps = cpg->eps;
    sw.precision = A.precision;
    int acc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) acc[q] = 0;
    long long* out = A.out + item.out_offset;
    __syncwarp();
#pragma unroll 1
    for (int pass = 0; pass < A.n_passes; ++pass) {
      const uint32_t pass_g = (uint32_t)(item.pass0 + pass);
#pragma unroll 1
      for (int c = 0; c < g.n_colors; ++c) {
#pragma unroll 1
        for (int e = g.color_start[c] + lane; e < g.color_start[c + 1]; e += 32) {
          const U32x4 x = philox4x32_10(U32x4{__ldg(g.site_l + e), pass_g, chain_id, SWEEP_TAG}, key0, key1);
          const uint32_t ent = __ldg(g.entries + e);
          int o;
          int F[B::NFEAT];
          sw.gather(ent, o, F);
          sw.decide(ent, philox_word(x, ent >> 30), x.y, o, F, acc);
        }
        __syncwarp();
      }
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) {
        const int v = warp_sum(acc[q]);
        if (lane == 0) out[(size_t)pass * NSLOT + q] = v;
        acc[q] = 0;
      }
    }
    for (int idx = lane; idx < L0 * L1 * L2; idx += 32) {
      const int i = idx % L0, j = (idx / L0) % L1, k = idx / (L0 * L1);
      const int pidx = (i + B::HALO) + PX * ((j + B::HALO) + PY * (k + B::HALO));
      gocc[i + (long long)L0 * (j + (long long)L1 * k)] = (int8_t)B::occ_of_code(s[pidx]);
    }
    __syncwarp();
  }
}

// Persistent pool kernel for chains too large for one CTA: each thread-block cluster of
// S CTAs takes chains from the work queue (rank 0 draws the item and writes it into every
// CTA's shared memory) and sweeps them as the batch kernel does (slabs, halo copies
// through distributed shared memory, split cluster barriers).  Per-pass outputs are
// accumulated with atomics (the host zeroes them).
template <class B, int NT>
__global__ void __launch_bounds__(NT, 1) ce_pool_cluster_kernel(const __grid_constant__ CePoolArgs<B::NFEAT> A) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  constexpr int PRE = (NS == 2) ? 3 : 1;
  extern __shared__ __align__(16) int8_t s[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];
  __shared__ int item_sm;
  cg::cluster_group cluster = cg::this_cluster();
  const int S = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int lane = threadIdx.x & 31;

#pragma unroll 1
  while (true) {
    if (rank == 0 && threadIdx.x == 0) {
      const int it = atomicAdd(A.next_item, 1);
      for (int r = 0; r < S; ++r) *cluster.map_shared_rank(&item_sm, (unsigned)r) = it;
    }
    cluster.sync();
    const int it = item_sm;
    if (it >= A.n_items) break;
    const PoolItem item = A.items[it];
    const PoolGeometry g = A.geoms[item.geom];
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int PX = L0 + 2 * B::HALO, PY = L1 + 2 * B::HALO, PXY = PX * PY;
    const int nkq = L2 / S, nkr = L2 % S;
    const int nk = nkq + (rank < nkr ? 1 : 0);
    const int k0 = rank * nkq + (rank < nkr ? rank : nkr);
    const int rprev = (rank + S - 1) % S;
    const int nk_prev = nkq + (rprev < nkr ? 1 : 0);
    int8_t* gocc = A.occ + item.occ_offset;
    for (int idx = threadIdx.x; idx < PXY * (nk + 2 * B::HALO); idx += NT) {
      const int ip = idx % PX, jp = (idx / PX) % PY, kp = idx / PXY;
      int i = ip - B::HALO, j = jp - B::HALO, k = k0 + kp - B::HALO;
      i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
      j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
      k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
      s[idx] = B::code_of_occ(gocc[i + (long long)L0 * (j + (long long)L1 * k)]);
    }
    if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;
    const CeChainParams* cpg = A.cp + item.param;
    load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
    const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
    const int* cstart = g.color_start + rank * (g.n_colors + 1);
    SiteSweeper<B> sw;
    sw.s = s;
    sw.s_prev = cluster.map_shared_rank(s, (unsigned)rprev);
    sw.s_next = cluster.map_shared_rank(s, (unsigned)((rank + 1) % S));
    sw.PX = PX;
    sw.PXY = PXY;
    sw.dI = L0;
    sw.dJ = L1 * PX;
    sw.dKp = nk_prev * PXY;
    sw.dKn = nk * PXY;
    sw.dmu32 = dmu32_sm;
    sw.dmu64 = dmu64_sm;
    sw.w = &A.w;
    sw.beta = cpg->beta;
    sw.beta_log2e = cpg->beta_log2e;
    sw.dtol = cpg->dtol;
    sw.eps = cpg->eps;
    sw.precision = A.precision;
    int acc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) acc[q] = 0;
    long long* out = A.out + item.out_offset;
    PhasePrefetch<PRE> pf;
    pf.template prepare<NT>(cstart, 0, g.entries, g.site_l, (uint32_t)item.pass0, chain_id, key0, key1);
    cluster.sync();
#pragma unroll 1
    for (int pass = 0; pass < A.n_passes; ++pass) {
      const uint32_t pass_g = (uint32_t)(item.pass0 + pass);
#pragma unroll 1
      for (int c = 0; c < g.n_colors; ++c) {
        sweep_phase<B, NT, PRE>(sw, pf, cstart, c, g.entries, g.site_l, pass_g, chain_id, key0, key1, acc);
        const bool last = (c + 1 == g.n_colors);
        cluster_arrive_release();
        pf.template prepare<NT>(cstart, last ? 0 : c + 1, g.entries, g.site_l, last ? pass_g + 1 : pass_g,
                                chain_id, key0, key1);
        cluster_wait_acquire();
        if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
          int* buf = acc_sm[(pass - 1) & 1];
          const int v = buf[threadIdx.x];
          buf[threadIdx.x] = 0;
          if (v)
            atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)(pass - 1) * NSLOT + threadIdx.x),
                      (unsigned long long)(long long)v);
        }
      }
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) {
        const int v = warp_sum(acc[q]);
        if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
        acc[q] = 0;
      }
    }
    cluster.sync();
    if (A.n_passes > 0 && threadIdx.x < NSLOT) {
      const int pl = A.n_passes - 1;
      const int v = acc_sm[pl & 1][threadIdx.x];
      if (v)
        atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)pl * NSLOT + threadIdx.x),
                  (unsigned long long)(long long)v);
    }
    for (int idx = threadIdx.x; idx < L0 * L1 * nk; idx += NT) {
      const int i = idx % L0, j = (idx / L0) % L1, kl = idx / (L0 * L1);
      const int pidx = (i + B::HALO) + PX * ((j + B::HALO) + PY * (kl + B::HALO));
      gocc[i + (long long)L0 * (j + (long long)L1 * (k0 + kl))] = (int8_t)B::occ_of_code(s[pidx]);
    }
    cluster.sync();
  }
}

// Persistent pool kernel over word-layout geometries (binary basis): as ce_pool_kernel
// (CLUSTER = false, one CTA per chain) or ce_pool_cluster_kernel (CLUSTER = true, S CTAs
// per chain), with the lattice held four sites per word (see ce_sweep_quad_kernel).
// Per-pass outputs are accumulated with atomics (the host zeroes them).
template <class B, int NT, bool CLUSTER, int MINB = 1>
__global__ void __launch_bounds__(NT, MINB) ce_pool_quad_kernel(const __grid_constant__ CePoolArgs<B::NFEAT> A) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  extern __shared__ __align__(16) uint32_t sq[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];
  __shared__ int item_sm;
  cg::cluster_group cluster = cg::this_cluster();
  const int S = CLUSTER ? (int)cluster.num_blocks() : 1;
  const int rank = CLUSTER ? (int)cluster.block_rank() : 0;
  const int lane = threadIdx.x & 31;
  auto sync_all = [&]() {
    if (CLUSTER)
      cluster.sync();
    else
      __syncthreads();
  };

#pragma unroll 1
  while (true) {
    if (rank == 0 && threadIdx.x == 0) {
      const int it = atomicAdd(A.next_item, 1);
      if (CLUSTER) {
        for (int r = 0; r < S; ++r) *cluster.map_shared_rank(&item_sm, (unsigned)r) = it;
      } else {
        item_sm = it;
      }
    }
    sync_all();
    const int it = item_sm;
    if (it >= A.n_items) break;
    const PoolItem item = A.items[it];
    const PoolGeometry g = A.geoms[item.geom];
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int Q = L0 / 4, RS = (Q + 2 * B::HALO) | 1, RY = L1 + 2 * B::HALO, RSY = RS * RY;
    const RowSlab sl = row_slab(L1, L2, S, rank, g.planes);
    const int rprev = (rank + S - 1) % S;
    int8_t* gocc = A.occ + item.occ_offset;
    load_word_window<B::HALO>(sq, gocc, L0, L1, L2, Q, RS, RY, sl.kb, sl.nk, threadIdx.x, NT);
    if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;
    const CeChainParams* cpg = A.cp + item.param;
    load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
    const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
    const int* cstart = g.color_start + rank * (g.n_colors + 1);
    QuadSweeper<B> sw;
    sw.s = sq;
    sw.s_prev = sq;
    sw.s_next = sq;
    if (CLUSTER) {
      sw.s_prev = cluster.map_shared_rank(sq, (unsigned)rprev);
      sw.s_next = cluster.map_shared_rank(sq, (unsigned)((rank + 1) % S));
    }
    sw.RS = RS;
    sw.RSY = RSY;
    sw.Q = Q;
    sw.dJ = L1 * RS;
    sw.dKp = sl.dkp * RSY;
    sw.dKn = sl.dkn * RSY;
    sw.rule = MetropolisRule<B>{dmu32_sm, dmu64_sm, &A.w, cpg->beta, cpg->beta_log2e, cpg->dtol, cpg->eps,
                                A.precision};
    int acc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) acc[q] = 0;
    long long* out = A.out + item.out_offset;
    QuadPrefetch pf;
    pf.template prepare<NT>(cstart, 0, g.entries, g.site_l, Q, (uint32_t)item.pass0, chain_id, key0, key1);
    sync_all();
#pragma unroll 1
    for (int pass = 0; pass < A.n_passes; ++pass) {
      const uint32_t pass_g = (uint32_t)(item.pass0 + pass);
#pragma unroll 1
      for (int c = 0; c < g.n_colors; ++c) {
        sweep_phase_quad<B, NT>(sw, pf, cstart, c, g.entries, g.site_l, pass_g, chain_id, key0, key1, acc);
        const bool last = (c + 1 == g.n_colors);
        if (CLUSTER) {
          cluster_arrive_release();
          pf.template prepare<NT>(cstart, last ? 0 : c + 1, g.entries, g.site_l, Q, last ? pass_g + 1 : pass_g,
                                  chain_id, key0, key1);
          cluster_wait_acquire();
        } else {
          pf.template prepare<NT>(cstart, last ? 0 : c + 1, g.entries, g.site_l, Q, last ? pass_g + 1 : pass_g,
                                  chain_id, key0, key1);
          __syncthreads();
        }
        if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
          int* buf = acc_sm[(pass - 1) & 1];
          const int v = buf[threadIdx.x];
          buf[threadIdx.x] = 0;
          if (v)
            atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)(pass - 1) * NSLOT + threadIdx.x),
                      (unsigned long long)(long long)v);
        }
      }
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) {
        const int v = warp_sum(acc[q]);
        if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
        acc[q] = 0;
      }
    }
    sync_all();
    if (A.n_passes > 0 && threadIdx.x < NSLOT) {
      const int pl = A.n_passes - 1;
      const int v = acc_sm[pl & 1][threadIdx.x];
      if (v)
        atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)pl * NSLOT + threadIdx.x),
                  (unsigned long long)(long long)v);
    }
    store_word_rows<B::HALO>(sq, gocc, L0, L1, Q, RS, RY, sl, threadIdx.x, NT);
    sync_all();
  }
}

// Persistent pool kernel of the ternary word layout: the work queue and phases of
// ce_pool_quad_kernel with the ternary sweeper (per-site Philox blocks, monomial counts).
template <int NFEAT, int NJ>
struct CeTPoolArgs {
  CePoolArgs<NFEAT> p;
  TernQuadWeights<NJ> tw;
};

template <class B, int NT, bool CLUSTER>
__global__ void __launch_bounds__(NT, 1)
    ce_pool_tquad_kernel(const __grid_constant__ CeTPoolArgs<B::NFEAT, B::NCOUNT> TA) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  const CePoolArgs<B::NFEAT>& A = TA.p;
  extern __shared__ __align__(16) uint32_t sq[];
  __shared__ int acc_sm[2][NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];
  __shared__ int item_sm;
  cg::cluster_group cluster = cg::this_cluster();
  const int S = CLUSTER ? (int)cluster.num_blocks() : 1;
  const int rank = CLUSTER ? (int)cluster.block_rank() : 0;
  const int lane = threadIdx.x & 31;
  auto sync_all = [&]() {
    if (CLUSTER)
      cluster.sync();
    else
      __syncthreads();
  };

#pragma unroll 1
  while (true) {
    if (rank == 0 && threadIdx.x == 0) {
      const int it = atomicAdd(A.next_item, 1);
      if (CLUSTER) {
        for (int r = 0; r < S; ++r) *cluster.map_shared_rank(&item_sm, (unsigned)r) = it;
      } else {
        item_sm = it;
      }
    }
    sync_all();
    const int it = item_sm;
    if (it >= A.n_items) break;
    const PoolItem item = A.items[it];
    const PoolGeometry g = A.geoms[item.geom];
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int Q = L0 / 4, RS = (Q + 2 * B::HALO) | 1, RY = L1 + 2 * B::HALO, RSY = RS * RY;
    const RowSlab sl = row_slab(L1, L2, S, rank, g.planes);
    const int rprev = (rank + S - 1) % S;
    int8_t* gocc = A.occ + item.occ_offset;
    load_word_window<B::HALO>(sq, gocc, L0, L1, L2, Q, RS, RY, sl.kb, sl.nk, threadIdx.x, NT);
    if (threadIdx.x < 2 * NSLOT) (&acc_sm[0][0])[threadIdx.x] = 0;
    const CeChainParams* cpg = A.cp + item.param;
    load_dmu<NS>(cpg, dmu32_sm, dmu64_sm);
    const uint32_t key0 = cpg->key0, key1 = cpg->key1, chain_id = cpg->chain_id;
    const int* cstart = g.color_start + rank * (g.n_colors + 1);
    TernQuadSweeper<B> sw;
    sw.s = sq;
    sw.s_prev = sq;
    sw.s_next = sq;
    if (CLUSTER) {
      sw.s_prev = cluster.map_shared_rank(sq, (unsigned)rprev);
      sw.s_next = cluster.map_shared_rank(sq, (unsigned)((rank + 1) % S));
    }
    sw.RS = RS;
    sw.RSY = RSY;
    sw.Q = Q;
    sw.dJ = L1 * RS;
    sw.dKp = sl.dkp * RSY;
    sw.dKn = sl.dkn * RSY;
    sw.rule = MetropolisRule<B>{dmu32_sm, dmu64_sm, &A.w, cpg->beta, cpg->beta_log2e, cpg->dtol, cpg->eps,
                                A.precision};
    sw.tw = &TA.tw;
    int acc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) acc[q] = 0;
    long long* out = A.out + item.out_offset;
    sync_all();
#pragma unroll 1
    for (int pass = 0; pass < A.n_passes; ++pass) {
      const uint32_t pass_g = (uint32_t)(item.pass0 + pass);
#pragma unroll 1
      for (int c = 0; c < g.n_colors; ++c) {
#pragma unroll 1
        for (int e = cstart[c] + threadIdx.x; e < cstart[c + 1]; e += NT)
          sw.update(__ldg(g.entries + e), __ldg(g.site_l + e), pass_g, chain_id, key0, key1, acc);
        sync_all();
        if (c == 0 && pass > 0 && threadIdx.x < NSLOT) {
          int* buf = acc_sm[(pass - 1) & 1];
          const int v = buf[threadIdx.x];
          buf[threadIdx.x] = 0;
          if (v)
            atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)(pass - 1) * NSLOT + threadIdx.x),
                      (unsigned long long)(long long)v);
        }
      }
#pragma unroll
      for (int q = 0; q < NSLOT; ++q) {
        const int v = warp_sum(acc[q]);
        if (lane == 0 && v) atomicAdd(&acc_sm[pass & 1][q], v);
        acc[q] = 0;
      }
    }
    sync_all();
    if (A.n_passes > 0 && threadIdx.x < NSLOT) {
      const int pl = A.n_passes - 1;
      const int v = acc_sm[pl & 1][threadIdx.x];
      if (v)
        atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)pl * NSLOT + threadIdx.x),
                  (unsigned long long)(long long)v);
    }
    store_word_rows<B::HALO>(sq, gocc, L0, L1, Q, RS, RY, sl, threadIdx.x, NT);
    sync_all();
  }
}

// ---- global-memory evaluation (per-proposal dE and full correlation sums)

struct GlobalLoader {
  const int8_t* occ;  // occupant indices of one chain
  int i, j, k, L0, L1, L2;
  int (*code)(int);
  __device__ __forceinline__ int idx(int di, int dj, int dk) const {
    int a = i + di, b = j + dj, c = k + dk;
    a = (a < 0) ? a + L0 : (a >= L0 ? a - L0 : a);
    b = (b < 0) ? b + L1 : (b >= L1 ? b - L1 : b);
    c = (c < 0) ? c + L2 : (c >= L2 ? c - L2 : c);
    return a + L0 * (b + L1 * c);
  }
};

template <class B>
struct GlobalCodeLoader {
  GlobalLoader g;
  __device__ __forceinline__ int operator()(int di, int dj, int dk) const {
    return B::code_of_occ(g.occ[g.idx(di, dj, dk)]);
  }
};

template <class B>
__global__ void ce_delta_e_kernel(CeWeights<B::NFEAT> w, const int8_t* occ, int L0, int L1, int L2,
                                  const CeChainParams* cp, const int* chain, const long long* sites,
                                  const int8_t* new_occ, long long n, double* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  constexpr int NS = B::NSPECIES;
  const long long N = (long long)L0 * L1 * L2;
  const int c = chain[t];
  const int8_t* o8 = occ + (size_t)c * N;
  const long long l = sites[t];
  const int i = (int)(l % L0), j = (int)((l / L0) % L1), k = (int)(l / ((long long)L0 * L1));
  GlobalCodeLoader<B> ld{GlobalLoader{o8, i, j, k, L0, L1, L2, nullptr}};
  int F[B::NFEAT];
  B::features(ld, F);
  const int o = o8[l], o2 = new_occ[t];
  double G64[B::NFUNC];
  for (int b = 0; b < B::NFUNC; ++b) G64[b] = 0.0;
  for (int k2 = 0; k2 < B::NFEAT; ++k2)
    G64[B::feat_b(k2)] = __dadd_rn(G64[B::feat_b(k2)], __dmul_rn(w.w64[k2], (double)F[k2]));
  double dE = 0.0;
  for (int b = 0; b < B::NFUNC; ++b)
    dE = __dadd_rn(dE, __dmul_rn((double)(B::psi(b, o2) - B::psi(b, o)), G64[b]));
  out[t] = __dsub_rn(dE, cp[c].dmu64[o * NS + o2]);
}

// Integer correlation sums of every class, recomputed from the occupation with the chain's
// planes staged in shared memory: CTA (x, chain) holds planes [x nk, x nk + nk) plus a
// HALO-plane border in k and a HALO border in i and j (periodic images), as occupant codes,
// so that every cluster member is a constant offset (out[chain][NCLASS], added atomically).
template <class B>
__global__ void __launch_bounds__(256) ce_corr_tiled_kernel(const int8_t* occ, int L0, int L1, int L2, int nk,
                                                            long long* out) {
  constexpr int H = B::HALO;
  constexpr int NC = B::NCLASS;
  extern __shared__ __align__(16) int8_t s[];
  const int chain = blockIdx.y;
  const int k0 = blockIdx.x * nk;
  const int nkb = min(nk, L2 - k0);
  const int PX = L0 + 2 * H, PY = L1 + 2 * H, PXY = PX * PY;
  const int8_t* g = occ + (size_t)chain * L0 * L1 * L2;
  // padded rows (PX bytes; row r = jp + PY kp of the window) by warps, four rows per step
  // so that four independent loads are in flight per lane; each row's lattice row and
  // periodic images found once.  Rows of 4-byte aligned length are read in 32-bit words
  // (the interior) plus the 2H halo bytes.
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, n_warps = blockDim.x >> 5;
  const int R = PY * (nkb + 2 * H);
  const bool vec = (L0 & 3) == 0 && (reinterpret_cast<uintptr_t>(g) & 3u) == 0;
  const int n_items = vec ? L0 / 4 + 2 * H : PX;  // per row: words + halo bytes, or bytes
  for (int r0 = 4 * warp; r0 < R; r0 += 4 * n_warps) {
    const int8_t* grow[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = min(r0 + u, R - 1);
      const int jp = r % PY, kp = r / PY;
      int j = jp - H, k = k0 + kp - H;
      j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
      k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
      grow[u] = g + (long long)L0 * (j + (long long)L1 * k);
    }
    for (int t = lane; t < n_items; t += 32) {
      // item t: a word of the interior (vec, t < L0/4), else one byte at padded position ip
      const bool word = vec && t < L0 / 4;
      int ip = t;
      if (vec && !word) ip = (t - L0 / 4 < H) ? t - L0 / 4 : L0 + (t - L0 / 4);
      int i = ip - H;
      i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
      uint32_t w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        w[u] = word ? __ldg(reinterpret_cast<const uint32_t*>(grow[u]) + t) : (uint32_t)(uint8_t)__ldg(grow[u] + i);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (r0 + u >= R) break;
        int8_t* srow = s + (size_t)(r0 + u) * PX;
        if (word) {
#pragma unroll
          for (int b = 0; b < 4; ++b) srow[H + 4 * t + b] = B::code_of_occ((int8_t)((w[u] >> (8 * b)) & 0xFFu));
        } else {
          srow[ip] = B::code_of_occ((int8_t)w[u]);
        }
      }
    }
  }
  __syncthreads();
  long long C[NC];
#pragma unroll
  for (int f = 0; f < NC; ++f) C[f] = 0;
  // the owned sites row by row (row rr = j + L1 kl)
  for (int rr = warp; rr < L1 * nkb; rr += n_warps) {
    const int j = rr % L1, kl = rr / L1;
    const int8_t* srow = s + H + PX * ((j + H) + PY * (kl + H));
    for (int i = lane; i < L0; i += 32) B::anchored(SmemLoader{srow + i, PX, PXY}, C);
  }
#pragma unroll
  for (int f = 0; f < NC; ++f) {
    long long v = C[f];
    for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o2);
    if ((threadIdx.x & 31) == 0 && v)
      atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)chain * NC + f), (unsigned long long)v);
  }
}

template <class B>
__global__ void ce_corr_kernel(const int8_t* occ, int L0, int L1, int L2, int n_chains, long long* out) {
  // grid: (blocks per chain, chains); out[chain][NCLASS]
  constexpr int NC = B::NCLASS;
  const int c = blockIdx.y;
  const long long N = (long long)L0 * L1 * L2;
  const int8_t* o8 = occ + (size_t)c * N;
  long long C[NC];
  for (int f = 0; f < NC; ++f) C[f] = 0;
  for (long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(l % L0), j = (int)((l / L0) % L1), k = (int)(l / ((long long)L0 * L1));
    GlobalCodeLoader<B> ld{GlobalLoader{o8, i, j, k, L0, L1, L2, nullptr}};
    B::anchored(ld, C);
  }
  for (int f = 0; f < NC; ++f) {
    long long v = C[f];
    for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o2);
    if ((threadIdx.x & 31) == 0 && v)
      atomicAdd(reinterpret_cast<unsigned long long*>(out + (size_t)c * NC + f), (unsigned long long)v);
  }
}

}  // namespace mg

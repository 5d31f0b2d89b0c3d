// Canonical (fixed-composition) Metropolis sweep of FCC cluster expansions: exchanges of
// occupants between pairs of same-colour sites.
//
// Correspondence with the reference: the canonical event of
// include/casm/monte/events/OccEventProposal.hh:108-237 (propose_canonical_event: a swap
// of two occupants of different species) accepted by methods/metropolis.hh:26-35 with the
// formation-energy change of the swap (occupation_metropolis.hh:114-150 drives such a loop
// with a user potential).  The reference draws one random swap per step; here a pass
// proposes, colour class by colour class, a perfect matching of the class's sites:
//
//   * Sites of one colour share no cluster, so the energy change of swapping i and j is
//     exactly dE_i(o_i -> o_j) + dE_j(o_j -> o_i), and the swaps of one phase touch disjoint
//     neighbourhoods: each is an independent Metropolis move.
//   * The matching of a phase pairs class positions k and (d - k) mod n (n sites in the
//     class in ascending site order; d drawn from Philox, independently of the state; a
//     fixed point k = d - k proposes nothing).  Every matching is an involution chosen
//     without looking at the state, so proposals are symmetric and detailed balance holds
//     for the phase; over phases every pair of a class is proposed.
//   * A colour class's composition is invariant under its swaps, so passes alternate
//     between two colourings (pass p uses colouring p & 1) whose classes connect every site
//     (checked on the host); atoms can then reach any site and the chain is ergodic at fixed
//     composition.
//
// Random numbers: Philox4x32-10 keyed by the chain's seed; the matching offset of (pass,
// colour) from counter (colour, pass, chain, CANON_D_TAG), word 0, d = (x * n) >> 32; the
// acceptance of a pair from counter (site index of its first site, pass, chain, CANON_TAG),
// word 0.  Decisions use the FP32 fast path of the sweep with the exact FP64 re-decision,
// the bounds widened for two sites (the host doubles the quantisation error and energy
// bound of the chain parameters).  One CTA per chain: the whole lattice with its periodic
// border is in shared memory, so a pair can join any two sites of a class.
#pragma once
#include "ce_sweep.cuh"

namespace mg {

constexpr uint32_t CANON_TAG = 0x4D434343u;    // acceptance draws of the canonical sweep
constexpr uint32_t CANON_D_TAG = 0x4D434344u;  // matching offsets of the canonical sweep

// one colouring's per-colour site lists (ascending site index within a colour)
struct CanonColouring {
  int n_colors;
  const int* color_start;   // [n_colors + 1]
  const uint32_t* entries;  // padded index | flags << 24
  const uint32_t* site_l;   // linear site index
};

template <int NFEAT>
struct CeCanonArgs {
  int L0, L1, L2, PX, PY;
  CanonColouring col[2];  // pass p uses col[p & 1]
  CeWeights<NFEAT> w;
  const CeChainParams* cp;  // [chain], exchange potentials zero
  int8_t* occ;              // [chain][N] occupant indices
  long long pass0;
  int n_passes;
  int n_chains;
  int precision;   // 0: FP64 decisions; 1: FP32 decisions (disagreements counted)
  long long* out;  // [n_passes][n_chains][NSLOT]: slot 0 accepted swaps
};

// FP64 change of formation energy of one site's flip (the fused order of MetropolisRule::exact)
template <class B>
__device__ __forceinline__ double site_de64(const CeWeights<B::NFEAT>& w, const int (&dpsi)[B::NFUNC],
                                            const int (&F)[B::NFEAT]) {
  double G64[B::NFUNC];
#pragma unroll
  for (int b = 0; b < B::NFUNC; ++b) G64[b] = 0.0;
#pragma unroll
  for (int k = 0; k < B::NFEAT; ++k) G64[B::feat_b(k)] = __fma_rn(w.w64[k], (double)F[k], G64[B::feat_b(k)]);
  double dE = 0.0;
#pragma unroll
  for (int b = 0; b < B::NFUNC; ++b) dE = __fma_rn((double)dpsi[b], G64[b], dE);
  return dE;
}

// Metropolis decision of the swap of the sites of entries ei and ej (same colour); on
// acceptance both sites and their copies are written and the correlation changes added.
template <class B>
__device__ __forceinline__ void canonical_swap(const SiteSweeper<B>& sw, uint32_t ei, uint32_t ej, uint32_t li,
                                               uint32_t pass, uint32_t chain_id, uint32_t key0, uint32_t key1,
                                               int (&acc)[CeSlots<B::NCLASS>::N]) {
  constexpr int NF = B::NFEAT, NC = B::NCLASS;
  int oi, oj;
  int Fi[NF], Fj[NF];
  sw.gather(ei, oi, Fi);
  sw.gather(ej, oj, Fj);
  if (oi == oj) return;  // the same species: nothing to exchange, no draw
  const U32x4 x = philox4x32_10(U32x4{li, pass, chain_id, CANON_TAG}, key0, key1);
  int dpi[B::NFUNC], dpj[B::NFUNC];
#pragma unroll
  for (int b = 0; b < B::NFUNC; ++b) {
    dpi[b] = B::psi(b, oj) - B::psi(b, oi);
    dpj[b] = -dpi[b];
  }
  const MetropolisRule<B> rule{sw.dmu32, sw.dmu64, sw.w, sw.beta, sw.beta_log2e, sw.dtol, sw.eps, sw.precision};
  // exact integer change of quantised energy (each part below 2^30 in magnitude)
  const int dEq = rule.dEq(dpi, [&](int k) { return Fi[k]; }) + rule.dEq(dpj, [&](int k) { return Fj[k]; });
  bool amb;
  bool accept = rule.fast(0, 0, dEq, x.x, amb);  // exchange potentials are zero
  if (amb) {
    const double dE = __dadd_rn(site_de64<B>(*sw.w, dpi, Fi), site_de64<B>(*sw.w, dpj, Fj));
    bool acc64;
    if (dE < 0.0) {
      acc64 = true;
    } else {
      const double u = __dmul_rn((double)x.x, 2.3283064365386962890625e-10);
      acc64 = u < exp(__dmul_rn(-dE, sw.beta));
    }
    acc[NC] += 1;
    if (sw.precision == 0) {
      accept = acc64;
    } else if (acc64 != accept) {
      acc[NC + 1] += 1;
    }
  }
  if (!accept) return;
  sw.store(ei, B::code_of_occ(oj));
  sw.store(ej, B::code_of_occ(oi));
  acc[0] += 1;
#pragma unroll
  for (int k = 0; k < NF; ++k) acc[B::feat_class(k)] += dpi[B::feat_b(k)] * Fi[k] + dpj[B::feat_b(k)] * Fj[k];
}

template <class B, int NT>
__global__ void __launch_bounds__(NT, 1) ce_canonical_kernel(const __grid_constant__ CeCanonArgs<B::NFEAT> A) {
  constexpr int NS = B::NSPECIES;
  constexpr int NSLOT = CeSlots<B::NCLASS>::N;
  extern __shared__ __align__(16) int8_t s[];
  __shared__ int acc_sm[NSLOT];
  __shared__ float dmu32_sm[NS * NS];
  __shared__ double dmu64_sm[NS * NS];

  const int chain = blockIdx.x;
  const int PX = A.PX, PY = A.PY, PXY = PX * PY;
  const int L0 = A.L0, L1 = A.L1, L2 = A.L2;
  const long long N = (long long)L0 * L1 * L2;
  int8_t* gocc = A.occ + (size_t)chain * N;

  // ---- the whole lattice with a HALO border on every side
  for (int idx = threadIdx.x; idx < PXY * (L2 + 2 * B::HALO); idx += NT) {
    const int ip = idx % PX, jp = (idx / PX) % PY, kp = idx / PXY;
    int i = ip - B::HALO, j = jp - B::HALO, k = kp - B::HALO;
    i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
    j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
    k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
    s[idx] = B::code_of_occ(gocc[i + (long long)L0 * (j + (long long)L1 * k)]);
  }
  if (threadIdx.x < NSLOT) acc_sm[threadIdx.x] = 0;

  const CeChainParams* cpg = A.cp + chain;
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
  sw.dKp = L2 * PXY;  // a plane k < HALO is also the upper border plane k + L2
  sw.dKn = L2 * PXY;  // a plane k >= L2 - HALO is also the lower border plane k - L2
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
  __syncthreads();

#pragma unroll 1
  for (int pass = 0; pass < A.n_passes; ++pass) {
    const uint32_t pass_g = (uint32_t)(A.pass0 + pass);
    const CanonColouring& cc = A.col[pass_g & 1u];
#pragma unroll 1
    for (int c = 0; c < cc.n_colors; ++c) {
      const int base = cc.color_start[c], n = cc.color_start[c + 1] - base;
      if (n >= 2) {
        const U32x4 xd = philox4x32_10(U32x4{(uint32_t)c, pass_g, chain_id, CANON_D_TAG}, key0, key1);
        const int d = (int)(((unsigned long long)xd.x * (unsigned long long)n) >> 32);
        // list entries of position k's pair (k < k2 only), fetched one pair ahead of its use
        auto fetch = [&](int k, uint32_t& ei, uint32_t& ej, uint32_t& li) -> bool {
          if (k >= n) return false;
          int k2 = d - k;
          if (k2 < 0) k2 += n;
          if (!(k < k2)) return false;
          ei = __ldg(cc.entries + base + k);
          ej = __ldg(cc.entries + base + k2);
          li = __ldg(cc.site_l + base + k);
          return true;
        };
        uint32_t ei = 0u, ej = 0u, li = 0u;
        bool cur = fetch(threadIdx.x, ei, ej, li);
#pragma unroll 1
        for (int k = threadIdx.x; k < n; k += NT) {
          uint32_t ei2 = 0u, ej2 = 0u, li2 = 0u;
          const bool nxt = fetch(k + NT, ei2, ej2, li2);
          if (cur) canonical_swap<B>(sw, ei, ej, li, pass_g, chain_id, key0, key1, acc);
          ei = ei2;
          ej = ej2;
          li = li2;
          cur = nxt;
        }
      }
      __syncthreads();
    }
    // this pass's counters: warps into shared memory, then one add per slot
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) {
      const int v = warp_sum(acc[q]);
      if (lane == 0 && v) atomicAdd(&acc_sm[q], v);
      acc[q] = 0;
    }
    __syncthreads();
    if (threadIdx.x < NSLOT) {
      const int v = acc_sm[threadIdx.x];
      acc_sm[threadIdx.x] = 0;
      if (v)
        atomicAdd(reinterpret_cast<unsigned long long*>(A.out + ((size_t)pass * A.n_chains + chain) * NSLOT +
                                                        threadIdx.x),
                  (unsigned long long)(long long)v);
    }
    __syncthreads();
  }

  // ---- write the lattice back
  for (long long l = threadIdx.x; l < N; l += NT) {
    const int i = (int)(l % L0), j = (int)((l / L0) % L1), k = (int)(l / ((long long)L0 * L1));
    gocc[l] = (int8_t)B::occ_of_code(s[(i + B::HALO) + PX * ((j + B::HALO) + PY * (k + B::HALO))]);
  }
}

}  // namespace mg

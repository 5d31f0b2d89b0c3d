// Rejection-free (N-fold way) semi-grand canonical dynamics of binary FCC cluster
// expansions: an event selector for the loop of include/casm/monte/methods/nfold.hh:48-149,
// run on the GPU.
//
// Events are single-site flips; the rate of flipping site l is the Metropolis acceptance
// probability min(1, exp(-beta dE_l)) (dE of the semi-grand canonical potential,
// basic_semigrand_canonical.hh:178-192).  An event is chosen with probability rate / R (R the
// total rate) and the state's residence time is -ln(u) / R: the N-fold way samples the
// Metropolis chain's equilibrium with time weights (nfold.hh: samples weighted by the time
// increment).  One CTA per chain holds the lattice, every site's rate (FP32) and a three-level
// tree of 32-wide sums (sites -> blocks of 32 -> superblocks of 1024 -> total); one warp
// selects an event by three warp-wide prefix scans.  After a flip the rates of the flipped
// site and of the 54 sites sharing a cluster with it are recomputed, then the sums of their
// blocks and superblocks, each from its children (no drift).  Integer correlation sums are
// tracked exactly; per pass of N events the kernel reports the pass's time, the total rate
// at its end and the time-weighted sums of the correlations.
//
// Random numbers: Philox4x32-10 keyed by the chain's seed, counter (event low, event high,
// chain, NFOLD_TAG): word 0 selects the event, word 1 draws its time increment.
#pragma once
#include "ce_sweep.cuh"

namespace mg {

constexpr uint32_t NFOLD_TAG = 0x4D434E46u;
constexpr int NFOLD_MAX_SUPER = 32;                     // superblocks of 1024 sites
constexpr int NFOLD_MAX_SITES = NFOLD_MAX_SUPER * 1024;  // 32768 sites per chain
constexpr int NFOLD_NOFF = 54;                          // sites sharing a cluster with a site

template <int NFEAT>
struct CeNfoldArgs {
  int L0, L1, L2, PX, PY;
  int n_super;  // superblocks: ceil(N / 1024)
  CeWeights<NFEAT> w;
  const CeChainParams* cp;  // [chain]
  int8_t* occ;              // [chain][N] occupant indices
  long long* corr;          // [chain][NCLASS] integer correlation sums (read, then written back)
  long long event0;         // events of each chain before this launch
  int n_passes;             // N events each
  int n_chains;
  double* out;              // [n_passes][n_chains][2 + NCLASS]: pass time, total rate at its end, sum dt corr_f
  int offs[3 * NFOLD_NOFF];  // the offsets (di, dj, dk) of the sites sharing a cluster with a site
};

// sum of v over a warp in a fixed order (every lane receives it)
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// inclusive prefix sum over a warp
__device__ __forceinline__ float warp_scan_f(float v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// The lane whose prefix interval holds `target` among 32 values v >= 0 (inclusive scan s):
// the first lane with v > 0 and s > target (a lane of zero value is never chosen, even when
// rounding made target slightly negative); when rounding leaves none, the last lane with
// v > 0 (lane 0 when all are zero).  *rest receives target less the values before it.
__device__ __forceinline__ int warp_pick(float v, float s, float target, int lane, float* rest) {
  const unsigned above = __ballot_sync(0xffffffffu, s > target && v > 0.f);
  int k;
  if (above) {
    k = __ffs(above) - 1;
  } else {
    const unsigned nz = __ballot_sync(0xffffffffu, v > 0.f);
    k = nz ? 31 - __clz(nz) : 0;
  }
  const float before = __shfl_sync(0xffffffffu, s - v, k);
  *rest = target - before;
  return k;
}

template <class B>
struct NfoldSite {
  const SiteSweeper<B>* sw;
  int L0, L1, L2, PX, PY;

  __device__ __forceinline__ uint32_t entry(int m) const {
    const int i = m % L0, j = (m / L0) % L1, k = m / (L0 * L1);
    uint32_t flags = 0;
    if (i < B::HALO) flags |= 1;
    else if (i >= L0 - B::HALO) flags |= 2;
    if (j < B::HALO) flags |= 4;
    else if (j >= L1 - B::HALO) flags |= 8;
    if (k < B::HALO) flags |= 16;
    if (k >= L2 - B::HALO) flags |= 32;
    return (uint32_t)((i + B::HALO) + PX * ((j + B::HALO) + PY * (k + B::HALO))) | (flags << 24);
  }

  // Metropolis rate of flipping site m: min(1, exp(-beta dE)) from the FP32 energy change
  __device__ __forceinline__ float rate(int m) const {
    int o;
    int F[B::NFEAT];
    sw->gather(entry(m), o, F);
    const int o2 = 1 - o;
    int dpsi[B::NFUNC];
#pragma unroll
    for (int b = 0; b < B::NFUNC; ++b) dpsi[b] = B::psi(b, o2) - B::psi(b, o);
    const MetropolisRule<B> rule{sw->dmu32, sw->dmu64, sw->w, sw->beta, sw->beta_log2e, sw->dtol, sw->eps,
                                 sw->precision};
    const int dEq = rule.dEq(dpsi, [&](int k) { return F[k]; });
    const float dE32 = fmaf((float)dEq, sw->w->qscale, -sw->dmu32[o * B::NSPECIES + o2]);
    return dE32 <= 0.f ? 1.f : fast_exp2(-dE32 * sw->beta_log2e);
  }

  __device__ __forceinline__ int neighbour(int m, int di, int dj, int dk) const {
    int i = m % L0 + di, j = (m / L0) % L1 + dj, k = m / (L0 * L1) + dk;
    i = (i % L0 + L0) % L0;
    j = (j % L1 + L1) % L1;
    k = (k % L2 + L2) % L2;
    return i + L0 * (j + L1 * k);
  }
};

// NT threads per chain, MINB chains resident per SM (the small instance keeps several chains
// of a small supercell on one SM, so that their sequential events overlap)
template <class B, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) ce_nfold_kernel(const __grid_constant__ CeNfoldArgs<B::NFEAT> A) {
  static_assert(B::NSPECIES == 2, "the rejection-free sweep flips binary sites");
  constexpr int NC = B::NCLASS;
  constexpr int NW = NT / 32;
  constexpr int NAFF = NFOLD_NOFF + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ float super_sum[NFOLD_MAX_SUPER];
  __shared__ long long corr_sm[NC];
  __shared__ double tw_sm[NC];
  __shared__ double time_sm;
  __shared__ float dt_sm, total_sm;
  __shared__ int sel_sm;
  __shared__ int aff[NAFF];
  __shared__ float dmu32_sm[4];
  __shared__ double dmu64_sm[4];

  const int chain = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int L0 = A.L0, L1 = A.L1, L2 = A.L2, PX = A.PX, PY = A.PY, PXY = PX * PY;
  const int N = L0 * L1 * L2, NPAD = A.n_super * 1024;
  float* rate = reinterpret_cast<float*>(smraw);  // [NPAD]
  float* block_sum = rate + NPAD;                  // [NPAD / 32]
  int8_t* s = reinterpret_cast<int8_t*>(block_sum + NPAD / 32);
  int8_t* gocc = A.occ + (size_t)chain * N;

  for (int idx = threadIdx.x; idx < PXY * (L2 + 2 * B::HALO); idx += NT) {
    const int ip = idx % PX, jp = (idx / PX) % PY, kp = idx / PXY;
    int i = ip - B::HALO, j = jp - B::HALO, k = kp - B::HALO;
    i = (i < 0) ? i + L0 : (i >= L0 ? i - L0 : i);
    j = (j < 0) ? j + L1 : (j >= L1 ? j - L1 : j);
    k = (k < 0) ? k + L2 : (k >= L2 ? k - L2 : k);
    s[idx] = B::code_of_occ(gocc[i + L0 * (j + L1 * k)]);
  }
  const CeChainParams* cpg = A.cp + chain;
  load_dmu<2>(cpg, dmu32_sm, dmu64_sm);
  if (threadIdx.x < NC) corr_sm[threadIdx.x] = A.corr[(size_t)chain * NC + threadIdx.x];
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
  sw.precision = 0;
  const NfoldSite<B> site{&sw, L0, L1, L2, PX, PY};
  __syncthreads();

  // ---- every site's rate, then the block and superblock sums
  for (int m = threadIdx.x; m < NPAD; m += NT) rate[m] = m < N ? site.rate(m) : 0.f;
  __syncthreads();
  for (int b = warp; b < NPAD / 32; b += NW) {
    const float v = warp_sum_f(rate[b * 32 + lane]);
    if (lane == 0) block_sum[b] = v;
  }
  __syncthreads();
  for (int q = warp; q < NFOLD_MAX_SUPER; q += NW) {
    const float v = q < A.n_super ? warp_sum_f(block_sum[q * 32 + lane]) : 0.f;
    if (lane == 0) super_sum[q] = v;
  }
  __syncthreads();

#pragma unroll 1
  for (int pass = 0; pass < A.n_passes; ++pass) {
    if (threadIdx.x < NC) tw_sm[threadIdx.x] = 0.0;
    if (threadIdx.x == 0) time_sm = 0.0;
    __syncthreads();
#pragma unroll 1
    for (int e = 0; e < N; ++e) {
      // 1. selection and time increment (warp 0)
      if (warp == 0) {
        const long long ev = A.event0 + (long long)pass * N + e;
        const U32x4 x = philox4x32_10(U32x4{(uint32_t)ev, (uint32_t)(ev >> 32), chain_id, NFOLD_TAG}, key0, key1);
        const float v1 = super_sum[lane];
        const float s1 = warp_scan_f(v1, lane);
        const float R = __shfl_sync(0xffffffffu, s1, 31);
        const float u = ((float)(x.x >> 8) + 0.5f) * 5.9604644775390625e-8f;  // (0, 1)
        float t;
        const int q = warp_pick(v1, s1, u * R, lane, &t);
        const float v2 = block_sum[q * 32 + lane];
        const int b = warp_pick(v2, warp_scan_f(v2, lane), t, lane, &t);
        const float v3 = rate[(q * 32 + b) * 32 + lane];
        const int k = warp_pick(v3, warp_scan_f(v3, lane), t, lane, &t);
        if (lane == 0) {
          // a leaf of positive rate is a site of the lattice; the bound is a guard only
          sel_sm = min((q * 32 + b) * 32 + k, N - 1);
          const float u2 = ((float)(x.y >> 8) + 1.0f) * 5.9604644775390625e-8f;  // (0, 1]
          dt_sm = -logf(u2) / R;
          total_sm = R;
        }
      }
      __syncthreads();
      // 2. thread 0: the residence time of the current state weights its correlation sums,
      // then the flip and its exact correlation change; the other threads: the sites the flip
      // affects (itself and the sites sharing a cluster with it)
      const int l = sel_sm;
      if (threadIdx.x > 0 && threadIdx.x <= NFOLD_NOFF)
        aff[threadIdx.x] = site.neighbour(l, A.offs[3 * (threadIdx.x - 1)], A.offs[3 * (threadIdx.x - 1) + 1],
                                          A.offs[3 * (threadIdx.x - 1) + 2]);
      if (threadIdx.x == 0) {
        aff[0] = l;
        const double dt = (double)dt_sm;
        time_sm += dt;
#pragma unroll
        for (int f = 0; f < NC; ++f) tw_sm[f] += dt * (double)corr_sm[f];
        const uint32_t ent = site.entry(l);
        int o;
        int F[B::NFEAT];
        sw.gather(ent, o, F);
        const int o2 = 1 - o;
        int dpsi[B::NFUNC];
#pragma unroll
        for (int bb = 0; bb < B::NFUNC; ++bb) dpsi[bb] = B::psi(bb, o2) - B::psi(bb, o);
#pragma unroll
        for (int kk = 0; kk < B::NFEAT; ++kk) corr_sm[B::feat_class(kk)] += dpsi[B::feat_b(kk)] * F[kk];
        sw.store(ent, B::code_of_occ(o2));
      }
      __syncthreads();
      // 3. new rates of the affected sites
      if (threadIdx.x < NAFF) rate[aff[threadIdx.x]] = site.rate(aff[threadIdx.x]);
      __syncthreads();
      // 4. their blocks' sums (a block met twice gets the same value twice)
      for (int a = warp; a < NAFF; a += NW) {
        const int bidx = aff[a] >> 5;
        const float v = warp_sum_f(rate[bidx * 32 + lane]);
        if (lane == 0) block_sum[bidx] = v;
      }
      __syncthreads();
      // 5. their superblocks' sums
      for (int a = warp; a < NAFF; a += NW) {
        const int q = aff[a] >> 10;
        const float v = warp_sum_f(block_sum[q * 32 + lane]);
        if (lane == 0) super_sum[q] = v;
      }
      __syncthreads();
    }
    // the pass's time, total rate and time-weighted correlation sums
    double* o = A.out + ((size_t)pass * A.n_chains + chain) * (2 + NC);
    if (threadIdx.x == 0) {
      o[0] = time_sm;
      float R = 0.f;
      for (int q = 0; q < NFOLD_MAX_SUPER; ++q) R += super_sum[q];
      o[1] = (double)R;
    }
    if (threadIdx.x < NC) o[2 + threadIdx.x] = tw_sm[threadIdx.x];
    __syncthreads();
  }

  // ---- the lattice and the correlation sums back
  for (int m = threadIdx.x; m < N; m += NT) {
    const int i = m % L0, j = (m / L0) % L1, k = m / (L0 * L1);
    gocc[m] = (int8_t)B::occ_of_code(s[(i + B::HALO) + PX * ((j + B::HALO) + PY * (k + B::HALO))]);
  }
  if (threadIdx.x < NC) A.corr[(size_t)chain * NC + threadIdx.x] = corr_sm[threadIdx.x];
}

}  // namespace mg

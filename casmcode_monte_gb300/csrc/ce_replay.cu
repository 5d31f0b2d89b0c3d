// Serial replay of the reference's semi-grand canonical Metropolis dynamics on an FCC
// cluster expansion, consuming the reference's own random-number sequence.
//
// One warp owns one chain.  It keeps the chain's occupation (int8 occupant indices,
// l = i + L0 (j + L1 k)) and the 312-word mt19937_64 state in shared memory, the occupant
// location lists of OccLocation in global memory, and replays step by step the loop of
// methods/occupation_metropolis.hh:114-150 with the proposal
// propose_semigrand_canonical_event (events/OccEventProposal.hh:260-336):
//
//   tsum[i+1] = tsum[i] + cand_size(swap[i].cand_a)      OccEventProposal.hh:277-289
//   r = random_real(tsum.back())                         :298 (uniform_real_distribution)
//   swap = first i with r < tsum[i+1]                    :300-304
//   l = loc[cand_a][random_int(cand_size - 1)]           OccLocation.hh:257-261 (choose_mol)
//   dE = dE_f(l: a -> b) - mu . N dx                     basic_semigrand_canonical.hh:178-192
//   accept: dE < 0, else random_real(1.0) < exp(-dE beta)  methods/metropolis.hh:26-35
//   apply: occ[l] = b; swap-remove l from loc[a], push it on loc[b]  OccLocation.cc:262-283
//
// The swaps are the semi-grand canonical swaps of one asymmetric unit in the reference's
// order (OccCandidate.cc:136-152): (a, b) for a = 0..ns-1, b = 0..ns-1, a != b.  The lists
// start in ascending site order per species, as OccLocation::initialize builds them
// (OccLocation.cc:39-115; one basis site, so mol id = site index).
//
// dE_f: the generated feature functions give exact integer changes dI_c of the class
// correlation sums; dE_f = sum over classes c >= 1, in class order, of
// V_c * ((dI_c * s_c) / M_c) in FP64 (s_c the class's site-basis scale, M_c its multiplicity),
// with explicit _rn intrinsics so that nothing is contracted.  For the binary occupation
// basis (s_c = 1) this equals, operation for operation, the clexulator-style sum of products
// of site functions.  random_int, random_real and generate_canonical follow libstdc++ over
// std::mt19937_64 (RandomNumberGenerator.hh:32-41).
//
// All lanes follow the same control flow on the same values; lane 0 alone writes shared and
// global memory, between __syncwarp()s; the lanes cooperate to regenerate the engine state.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/montegpu.h"
#include "ce_host.cuh"
#include "mg_common.cuh"

namespace mg {

template <int NC>
struct CeReplayWeights {
  double v[NC];     // ECI per class
  double s[NC];     // site-basis scale of the class (product over its decoration)
  double mult[NC];  // multiplicity per primitive cell
};

struct CeReplayArgs {
  int L0, L1, L2, n_chains;
  int n_passes;
  const double* beta;   // [chain]
  const double* mu;     // [chain][CE_MAX_SPECIES - 1]
  int8_t* occ;          // [chain][N]
  int32_t* loc;         // [chain][NSPECIES][N] occupant lists
  int32_t* pos;         // [chain][N] position of each site in its species' list
  int32_t* nloc;        // [chain][NSPECIES] list sizes
  uint64_t* mt;         // [chain][313]: 312 words + position
  unsigned long long* n_accept;  // [chain] running totals
  unsigned long long* n_reject;  // [chain]
  long long* out;       // [n_passes][n_chains][NCLASS + 2] or null
  int* status;          // [chain]: 0 ok, 1 no swap chosen (the reference throws), 2 lists corrupt
};

template <class B>
__global__ void __launch_bounds__(32) ce_replay_kernel(CeReplayWeights<B::NCLASS> w, CeReplayArgs P) {
  constexpr int NS = B::NSPECIES;
  constexpr int NC = B::NCLASS;
  constexpr int NSWAP = NS * (NS - 1);
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* x = reinterpret_cast<uint64_t*>(smem);
  int8_t* occ = reinterpret_cast<int8_t*>(smem + MT_N * sizeof(uint64_t));
  const int chain = blockIdx.x;
  const int lane = threadIdx.x;
  const int L0 = P.L0, L1 = P.L1, L2 = P.L2;
  const int N = L0 * L1 * L2;
  int8_t* gocc = P.occ + (size_t)chain * N;
  uint64_t* gmt = P.mt + (size_t)chain * (MT_N + 1);
  int32_t* loc = P.loc + (size_t)chain * NS * N;
  int32_t* pos = P.pos + (size_t)chain * N;
  for (int i = lane; i < N; i += 32) occ[i] = gocc[i];
  for (int i = lane; i < MT_N; i += 32) x[i] = gmt[i];
  int p = (int)gmt[MT_N];
  int n[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) n[s] = P.nloc[(size_t)chain * NS + s];
  __syncwarp();

  const double beta = P.beta[chain];
  double mu[NS - 1];
#pragma unroll
  for (int i = 0; i < NS - 1; ++i) mu[i] = P.mu[(size_t)chain * (CE_MAX_SPECIES - 1) + i];
  unsigned long long n_acc = P.n_accept[chain], n_rej = P.n_reject[chain];
  int status = 0;

#pragma unroll 1
  for (int pass = 0; pass < P.n_passes && !status; ++pass) {
    long long dcorr[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) dcorr[c] = 0;
    long long pass_acc = 0, pass_rej = 0;
#pragma unroll 1
    for (int step = 0; step < N; ++step) {
      // choose the swap type: cumulative candidate counts, first partial sum above r
      double tsum[NSWAP + 1];
      tsum[0] = 0.0;
      int sa[NSWAP], sb[NSWAP];
      {
        int i = 0;
#pragma unroll
        for (int a = 0; a < NS; ++a)
#pragma unroll
          for (int b = 0; b < NS; ++b)
            if (a != b) {
              sa[i] = a;
              sb[i] = b;
              tsum[i + 1] = __dadd_rn(tsum[i], (double)n[a]);
              ++i;
            }
      }
      const double u0 = mt_canonical_warp(x, p, lane);
      const double r = __dadd_rn(__dmul_rn(u0, tsum[NSWAP]), 0.0);
      int k = -1;
#pragma unroll
      for (int i = NSWAP - 1; i >= 0; --i)
        if (r < tsum[i + 1]) k = i;
      if (k < 0) {
        status = 1;
        break;
      }
      int a = 0, b = 0;
#pragma unroll
      for (int i = 0; i < NSWAP; ++i)
        if (i == k) {
          a = sa[i];
          b = sb[i];
        }
      int na = 0;
#pragma unroll
      for (int s = 0; s < NS; ++s)
        if (s == a) na = n[s];
      if (na < 1) {
        status = 1;
        break;
      }
      const uint64_t idx = mt_uniform_int_warp(x, p, lane, (uint64_t)na);
      const int l = loc[(size_t)a * N + (int)idx];
      if (l < 0 || l >= N || occ[l] != a) {  // lists out of step with the occupation
        status = 2;
        break;
      }
      // exact integer change of every class correlation sum
      const int i0 = l % L0, j0 = (l / L0) % L1, k0 = l / (L0 * L1);
      GlobalCodeLoader<B> ld{GlobalLoader{occ, i0, j0, k0, L0, L1, L2, nullptr}};
      int F[B::NFEAT];
      B::features(ld, F);
      long long dI[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) dI[c] = 0;
#pragma unroll
      for (int f = 0; f < B::NFEAT; ++f)
        dI[B::feat_class(f)] += (long long)(B::psi(B::feat_b(f), b) - B::psi(B::feat_b(f), a)) * F[f];
      double dEf = 0.0;
#pragma unroll
      for (int c = 1; c < NC; ++c)
        dEf = __dadd_rn(dEf, __dmul_rn(w.v[c], __ddiv_rn(__dmul_rn((double)dI[c], w.s[c]), w.mult[c])));
      double mdx = 0.0;
#pragma unroll
      for (int i = 0; i < NS - 1; ++i) {
        const double d = (b == i + 1 ? 1.0 : 0.0) - (a == i + 1 ? 1.0 : 0.0);
        mdx = __dadd_rn(mdx, __dmul_rn(mu[i], d));
      }
      const double dE = __dsub_rn(dEf, mdx);
      bool accept = true;
      if (!(dE < 0.0)) {
        const double u1 = __dadd_rn(__dmul_rn(mt_canonical_warp(x, p, lane), 1.0), 0.0);
        accept = u1 < exp(__dmul_rn(-dE, beta));
      }
      if (accept) {
        ++n_acc;
        ++pass_acc;
#pragma unroll
        for (int c = 0; c < NC; ++c) dcorr[c] += dI[c];
        int nb = 0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
          if (s == b) nb = n[s];
        __syncwarp();
        if (lane == 0) {
          occ[l] = (int8_t)b;
          const int pl = pos[l];
          const int back = loc[(size_t)a * N + na - 1];
          loc[(size_t)a * N + pl] = back;
          pos[back] = pl;
          pos[l] = nb;
          loc[(size_t)b * N + nb] = l;
        }
        __syncwarp();
#pragma unroll
        for (int s = 0; s < NS; ++s) n[s] += (s == b) - (s == a);
      } else {
        ++n_rej;
        ++pass_rej;
      }
    }
    if (P.out && lane == 0) {
      long long* o = P.out + ((size_t)pass * P.n_chains + chain) * (NC + 2);
      o[0] = pass_acc;
#pragma unroll
      for (int c = 1; c < NC; ++c) o[c] = dcorr[c];
      o[NC] = pass_rej;
      o[NC + 1] = status;
    }
  }
  __syncwarp();
  for (int i = lane; i < N; i += 32) gocc[i] = occ[i];
  for (int i = lane; i < MT_N; i += 32) gmt[i] = x[i];
  if (lane == 0) {
    gmt[MT_N] = (uint64_t)p;
#pragma unroll
    for (int s = 0; s < NS; ++s) P.nloc[(size_t)chain * NS + s] = n[s];
    P.n_accept[chain] = n_acc;
    P.n_reject[chain] = n_rej;
    P.status[chain] = status;
  }
}

}  // namespace mg

// ---------------------------------------------------------------- C-ABI
struct mg_ce_replay {
  const mg_ce_model* model = nullptr;
  int L0 = 0, L1 = 0, L2 = 0, n_chains = 0;
  long long N = 0;
  long long n_pass = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  double *dbeta = nullptr, *dmu = nullptr;
  int8_t* docc = nullptr;
  int32_t *dloc = nullptr, *dpos = nullptr, *dnloc = nullptr;
  uint64_t* dmt = nullptr;
  unsigned long long *dacc = nullptr, *drej = nullptr;
  long long* dout = nullptr;
  size_t out_cap = 0;
  int* dstatus = nullptr;
  size_t smem = 0;
};

namespace {

void free_ce_replay(mg_ce_replay* h) {
  if (!h) return;
  cudaFree(h->dbeta);
  cudaFree(h->dmu);
  cudaFree(h->docc);
  cudaFree(h->dloc);
  cudaFree(h->dpos);
  cudaFree(h->dnloc);
  cudaFree(h->dmt);
  cudaFree(h->dacc);
  cudaFree(h->drej);
  cudaFree(h->dout);
  cudaFree(h->dstatus);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

template <class B>
void fill_replay_weights(const mg_ce_model* m, mg::CeReplayWeights<B::NCLASS>& w) {
  for (int c = 0; c < B::NCLASS; ++c) {
    w.v[c] = m->eci[c];
    w.s[c] = m->scale[c];
    w.mult[c] = (double)m->mult[c];
  }
}

template <class B>
cudaError_t launch_replay(const mg_ce_replay* h, const mg::CeReplayArgs& a) {
  mg::CeReplayWeights<B::NCLASS> w;
  fill_replay_weights<B>(h->model, w);
  static bool attr_set[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (h->smem > 48 * 1024 && dev >= 0 && dev < 64 && !attr_set[dev]) {
    e = cudaFuncSetAttribute(mg::ce_replay_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) return e;
    attr_set[dev] = true;
  }
  mg::ce_replay_kernel<B><<<h->n_chains, 32, h->smem, h->stream>>>(w, a);
  return cudaGetLastError();
}

constexpr long long kMaxReplaySites = 200000;

}  // namespace

extern "C" {

int mg_ce_replay_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains, const double* temperature,
                        const double* mu, const int8_t* occ, const char* const* engine_states,
                        mg_ce_replay** out) {
  if (!m || !out || !temperature || !occ || !engine_states || n_chains < 1 || (m->n_species > 1 && !mu)) {
    mg::set_error("Error in mg_ce_replay_create: invalid argument");
    return MG_ERR_INVALID;
  }
  if (L0 < 4 || L1 < 4 || L2 < 4) {
    mg::set_error("Error in mg_ce_replay_create: supercell dimensions must be >= 4 (cluster images overlap)");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  if (N > kMaxReplaySites) {
    mg::set_error("Error in mg_ce_replay_create: supercell exceeds 200000 sites (shared-memory replay)");
    return MG_ERR_INVALID;
  }
  const int ns = m->n_species;
  for (long long i = 0; i < N * n_chains; ++i)
    if (occ[i] < 0 || occ[i] >= ns) {
      mg::set_error("Error in mg_ce_replay_create: occupant index out of range");
      return MG_ERR_INVALID;
    }
  for (int c = 0; c < n_chains; ++c)
    if (!(temperature[c] > 0.0)) {
      mg::set_error("Error in mg_ce_replay_create: temperature must be > 0");
      return MG_ERR_INVALID;
    }
  std::vector<uint64_t> mt((size_t)n_chains * (mg::MT_N + 1));
  for (int c = 0; c < n_chains; ++c)
    if (!engine_states[c] || mg::parse_mt_state(engine_states[c], mt.data() + (size_t)c * (mg::MT_N + 1)) ||
        mt[(size_t)c * (mg::MT_N + 1) + mg::MT_N] > (uint64_t)mg::MT_N) {
      mg::set_error("Error in mg_ce_replay_create: malformed engine state");
      return MG_ERR_INVALID;
    }
  // occupant lists as OccLocation::initialize builds them: ascending site order per species
  std::vector<int32_t> loc((size_t)n_chains * ns * N, 0), pos((size_t)n_chains * N), nloc((size_t)n_chains * ns, 0);
  for (int c = 0; c < n_chains; ++c)
    for (long long l = 0; l < N; ++l) {
      const int s = occ[(size_t)c * N + l];
      int32_t& n = nloc[(size_t)c * ns + s];
      pos[(size_t)c * N + l] = n;
      loc[((size_t)c * ns + s) * N + n] = (int32_t)l;
      ++n;
    }
  const double KB = 8.6173303E-05;
  std::vector<double> beta(n_chains), mu_pad((size_t)n_chains * (mg::CE_MAX_SPECIES - 1), 0.0);
  for (int c = 0; c < n_chains; ++c) {
    beta[c] = 1.0 / (KB * temperature[c]);
    for (int i = 0; i < ns - 1; ++i) mu_pad[(size_t)c * (mg::CE_MAX_SPECIES - 1) + i] = mu[(size_t)c * (ns - 1) + i];
  }
  auto* h = new mg_ce_replay();
  h->model = m;
  h->L0 = L0;
  h->L1 = L1;
  h->L2 = L2;
  h->N = N;
  h->n_chains = n_chains;
  h->smem = sizeof(uint64_t) * mg::MT_N + (size_t)((N + 15) / 16) * 16;
  auto fail = [&](cudaError_t e, const char* what) {
    mg::set_error(std::string("CUDA error in mg_ce_replay_create: ") + what + ": " + cudaGetErrorString(e));
    free_ce_replay(h);
    return MG_ERR_CUDA;
  };
  cudaError_t e;
#define MGX(expr, what) \
  if ((e = (expr)) != cudaSuccess) return fail(e, what)
  MGX(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
  MGX(cudaEventCreate(&h->ev0), "event");
  MGX(cudaEventCreate(&h->ev1), "event");
  MGX(cudaMalloc(&h->dbeta, sizeof(double) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dmu, sizeof(double) * mu_pad.size()), "malloc");
  MGX(cudaMalloc(&h->docc, (size_t)N * n_chains), "malloc");
  MGX(cudaMalloc(&h->dloc, sizeof(int32_t) * loc.size()), "malloc");
  MGX(cudaMalloc(&h->dpos, sizeof(int32_t) * pos.size()), "malloc");
  MGX(cudaMalloc(&h->dnloc, sizeof(int32_t) * nloc.size()), "malloc");
  MGX(cudaMalloc(&h->dmt, sizeof(uint64_t) * mt.size()), "malloc");
  MGX(cudaMalloc(&h->dacc, sizeof(unsigned long long) * n_chains), "malloc");
  MGX(cudaMalloc(&h->drej, sizeof(unsigned long long) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dstatus, sizeof(int) * n_chains), "malloc");
  MGX(cudaMemcpyAsync(h->dbeta, beta.data(), sizeof(double) * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dmu, mu_pad.data(), sizeof(double) * mu_pad.size(), cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->docc, occ, (size_t)N * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dloc, loc.data(), sizeof(int32_t) * loc.size(), cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dpos, pos.data(), sizeof(int32_t) * pos.size(), cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dnloc, nloc.data(), sizeof(int32_t) * nloc.size(), cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dmt, mt.data(), sizeof(uint64_t) * mt.size(), cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemsetAsync(h->dacc, 0, sizeof(unsigned long long) * n_chains, h->stream), "memset");
  MGX(cudaMemsetAsync(h->drej, 0, sizeof(unsigned long long) * n_chains, h->stream), "memset");
  MGX(cudaMemsetAsync(h->dstatus, 0, sizeof(int) * n_chains, h->stream), "memset");
  MGX(cudaStreamSynchronize(h->stream), "sync");
#undef MGX
  *out = h;
  return MG_OK;
}

int mg_ce_replay_run(mg_ce_replay* h, int n_passes, long long* out) {
  if (!h || n_passes < 0) {
    mg::set_error("Error in mg_ce_replay_run: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n_passes == 0) return MG_OK;
  const int nslot = h->model->n_classes + 2;
  const size_t need = (size_t)n_passes * h->n_chains * nslot;
  if (out && need > h->out_cap) {
    cudaFree(h->dout);
    h->dout = nullptr;
    MG_CUDA_TRY(cudaMalloc(&h->dout, sizeof(long long) * need));
    h->out_cap = need;
  }
  mg::CeReplayArgs a{h->L0, h->L1, h->L2, h->n_chains, n_passes, h->dbeta, h->dmu, h->docc, h->dloc, h->dpos,
                     h->dnloc, h->dmt, h->dacc, h->drej, out ? h->dout : nullptr, h->dstatus};
  MG_CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  MG_CUDA_TRY(h->model->kind == 0 ? launch_replay<mg::FccBinary>(h, a) : launch_replay<mg::FccTernary>(h, a));
  MG_CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
  if (out) MG_CUDA_TRY(cudaMemcpyAsync(out, h->dout, sizeof(long long) * need, cudaMemcpyDeviceToHost, h->stream));
  std::vector<int> status(h->n_chains);
  MG_CUDA_TRY(cudaMemcpyAsync(status.data(), h->dstatus, sizeof(int) * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  for (int c = 0; c < h->n_chains; ++c) {
    if (status[c] == 1) {
      mg::set_error("Error in choose_semigrand_canonical_swap");
      return MG_ERR_INVALID;
    }
    if (status[c]) {
      mg::set_error("Error in OccLocation::apply: species mismatch");
      return MG_ERR_INVALID;
    }
  }
  h->n_pass += n_passes;
  return MG_OK;
}

int mg_ce_replay_get_occ(mg_ce_replay* h, int8_t* occ) {
  if (!h || !occ) {
    mg::set_error("Error in mg_ce_replay_get_occ: invalid argument");
    return MG_ERR_INVALID;
  }
  MG_CUDA_TRY(cudaMemcpyAsync(occ, h->docc, (size_t)h->N * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return MG_OK;
}

int mg_ce_replay_engine_state(mg_ce_replay* h, int chain, char* buf, int buf_len) {
  if (!h || chain < 0 || chain >= h->n_chains || !buf || buf_len < 1) {
    mg::set_error("Error in mg_ce_replay_engine_state: invalid argument");
    return MG_ERR_INVALID;
  }
  uint64_t s[mg::MT_N + 1];
  MG_CUDA_TRY(cudaMemcpyAsync(s, h->dmt + (size_t)chain * (mg::MT_N + 1), sizeof(s), cudaMemcpyDeviceToHost,
                              h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  const std::string t = mg::format_mt_state(s);
  if ((int)t.size() + 1 > buf_len) {
    mg::set_error("Error in mg_ce_replay_engine_state: buffer too small");
    return MG_ERR_INVALID;
  }
  std::memcpy(buf, t.c_str(), t.size() + 1);
  return MG_OK;
}

int mg_ce_replay_candidates(mg_ce_replay* h, int chain, int32_t* sizes, int32_t* sites) {
  if (!h || chain < 0 || chain >= h->n_chains || !sizes || !sites) {
    mg::set_error("Error in mg_ce_replay_candidates: invalid argument");
    return MG_ERR_INVALID;
  }
  const int ns = h->model->n_species;
  MG_CUDA_TRY(cudaMemcpyAsync(sizes, h->dnloc + (size_t)chain * ns, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost,
                              h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  long long off = 0;
  for (int s = 0; s < ns; ++s) {
    if (sizes[s] < 0 || off + sizes[s] > h->N) {
      mg::set_error("Error in mg_ce_replay_candidates: corrupt occupant lists");
      return MG_ERR_INVALID;
    }
    if (sizes[s] > 0)
      MG_CUDA_TRY(cudaMemcpyAsync(sites + off, h->dloc + ((size_t)chain * ns + s) * h->N, sizeof(int32_t) * sizes[s],
                                  cudaMemcpyDeviceToHost, h->stream));
    off += sizes[s];
  }
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return MG_OK;
}

int mg_ce_replay_counts(mg_ce_replay* h, unsigned long long* n_accept, unsigned long long* n_reject) {
  if (!h || !n_accept || !n_reject) {
    mg::set_error("Error in mg_ce_replay_counts: invalid argument");
    return MG_ERR_INVALID;
  }
  MG_CUDA_TRY(cudaMemcpyAsync(n_accept, h->dacc, sizeof(unsigned long long) * h->n_chains, cudaMemcpyDeviceToHost,
                              h->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(n_reject, h->drej, sizeof(unsigned long long) * h->n_chains, cudaMemcpyDeviceToHost,
                              h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return MG_OK;
}

int mg_ce_replay_last_kernel_ms(const mg_ce_replay* h, float* ms) {
  if (!h || !ms) {
    mg::set_error("Error in mg_ce_replay_last_kernel_ms: invalid argument");
    return MG_ERR_INVALID;
  }
  *ms = h->last_ms;
  return MG_OK;
}

int mg_ce_replay_destroy(mg_ce_replay* h) {
  free_ce_replay(h);
  return MG_OK;
}

}  // extern "C"

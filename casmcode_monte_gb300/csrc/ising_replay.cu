// Serial-replay semi-grand canonical Metropolis for the 2-D Ising model, bit-exact with
// the reference's CPU loop.
//
// One warp owns one chain.  It keeps the chain's occupation (int8, column-major
// l = rows*j + i as IsingConfiguration, ising_cpp/model.hh:93-99) and the 312-word
// mt19937_64 state in shared memory and replays, step by step:
//   propose  l = uniform_int(0, N-1)            basic_semigrand_canonical.hh:308-315
//   dE_f = (-J * (new - old)) * (sum of 4 nbrs) model.hh:309-314
//   dE   = dE_f - mu * ((new - old) / 2.0)      basic_semigrand_canonical.hh:178-192,
//                                               model.hh:425-435
//   accept dE < 0, else u < exp(-dE * beta)     metropolis.hh:26-35
//   n_pass bookkeeping, sample every sample_period passes
//                                               basic_occupation_metropolis.hh:381-421
// All lanes execute the same uniform control flow (values are broadcast from shared
// memory); the lanes cooperate only to regenerate the mt19937_64 state and to compute
// the per-sample row/column dot products.  Floating-point steps use explicit _rn
// intrinsics so that no multiply-add is contracted.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/montegpu.h"
#include "mg_common.cuh"

namespace mg {

struct IsingReplayParams {
  int rows, cols, n_chains;
  int use_nlist;
  int sample_period;
  long long pass0;  // pass count at chunk start (for sample scheduling)
  int n_passes;
  int max_samples;  // capacity of the sample buffer per chain
  const double* J;     // [chain]
  const double* mu;    // [chain]
  const double* beta;  // [chain]
  int8_t* occ;         // [chain][N]
  uint64_t* mt;        // [chain][313]: 312 words + index
  long long* spin_sum;  // [chain] running sum of s
  long long* bond_sum;  // [chain] running sum over bonds of s_a s_b
  unsigned long long* n_accept;  // [chain]
  unsigned long long* n_reject;  // [chain]
  long long* samples;  // [chain][max_samples][2 + rows + cols]
  int* n_samples;      // [chain] samples written this chunk
  int* status;         // [chain] nonzero on error
};

__device__ __forceinline__ uint64_t mt_next(uint64_t* x, int& p, int lane) {
  if (p >= MT_N) {
    mt_twist_warp(x, lane);
    p = 0;
  }
  const uint64_t y = x[p];
  p += 1;
  return mt_temper(y);
}

__global__ void __launch_bounds__(32) ising_replay_kernel(IsingReplayParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* x = reinterpret_cast<uint64_t*>(smem);
  int8_t* occ = reinterpret_cast<int8_t*>(smem + MT_N * sizeof(uint64_t));
  const int chain = blockIdx.x;
  const int lane = threadIdx.x;
  const int rows = P.rows, cols = P.cols;
  const int N = rows * cols;
  const int8_t* gocc = P.occ + (size_t)chain * N;
  uint64_t* gmt = P.mt + (size_t)chain * (MT_N + 1);
  for (int i = lane; i < N; i += 32) occ[i] = gocc[i];
  for (int i = lane; i < MT_N; i += 32) x[i] = gmt[i];
  int p = (int)gmt[MT_N];
  __syncwarp();

  const double J = P.J[chain], mu = P.mu[chain], beta = P.beta[chain];
  const double negJ = -J;
  long long spin_sum = P.spin_sum[chain];
  long long bond_sum = P.bond_sum[chain];
  unsigned long long n_acc = P.n_accept[chain], n_rej = P.n_reject[chain];
  // uniform_int_distribution<long>(0, N-1): Lemire with range N
  const uint64_t range = (uint64_t)N;
  const uint64_t threshold = (0ull - range) % range;
  const int stride = 2 + rows + cols;
  int ns = 0;

#pragma unroll 1
  for (int pass = 0; pass < P.n_passes; ++pass) {
#pragma unroll 1
    for (int step = 0; step < N; ++step) {
      uint64_t w = mt_next(x, p, lane);
      uint64_t lo = w * range;
      uint64_t hi = __umul64hi(w, range);
      if (lo < range) {
        while (lo < threshold) {
          w = mt_next(x, p, lane);
          lo = w * range;
          hi = __umul64hi(w, range);
        }
      }
      const int l = (int)hi;
      const int i = l % rows, j = l / rows;
      const int o = occ[l];
      const int nw = -o;
      const int ip = (i + 1 == rows) ? 0 : i + 1, im = (i == 0) ? rows - 1 : i - 1;
      const int jp = (j + 1 == cols) ? 0 : j + 1, jm = (j == 0) ? cols - 1 : j - 1;
      const int s4 = occ[ip + rows * j] + occ[i + rows * jp] + occ[im + rows * j] + occ[i + rows * jm];
      const double dEf = __dmul_rn(__dmul_rn(negJ, (double)(nw - o)), (double)s4);
      const double Ndx = __dmul_rn((double)(nw - o), 0.5);
      const double dE = __dsub_rn(dEf, __dmul_rn(mu, Ndx));
      bool accept;
      if (dE < 0.0) {
        accept = true;
      } else {
        // std::generate_canonical<double, 53>(mt19937_64): double(word) / 2^64, < 1
        const uint64_t w2 = mt_next(x, p, lane);
        double u = __dmul_rn(__ull2double_rn(w2), 5.421010862427522170e-20);
        if (u >= 1.0) u = 0.99999999999999988898;  // nextafter(1, 0)
        const double prob = exp(__dmul_rn(-dE, beta));
        accept = u < prob;
      }
      if (accept) {
        ++n_acc;
        __syncwarp();
        if (lane == 0) occ[l] = (int8_t)nw;
        spin_sum += nw - o;
        bond_sum += (long long)(nw - o) * s4;
        __syncwarp();
      } else {
        ++n_rej;
      }
    }
    const long long pass_count = P.pass0 + pass + 1;
    if (pass_count % P.sample_period == 0) {
      if (ns < P.max_samples) {
        long long* out = P.samples + ((size_t)chain * P.max_samples + ns) * stride;
        if (lane == 0) {
          out[0] = spin_sum;
          out[1] = bond_sum;
        }
        if (!P.use_nlist) {
          // row dot products sum_j s(i,j) s(i+1,j) and column dots sum_i s(i,j) s(i,j+1)
          for (int r = lane; r < rows; r += 32) {
            const int rn = (r + 1 == rows) ? 0 : r + 1;
            long long d = 0;
            for (int c = 0; c < cols; ++c) d += (long long)occ[r + rows * c] * occ[rn + rows * c];
            out[2 + r] = d;
          }
          for (int c = lane; c < cols; c += 32) {
            const int cn = (c + 1 == cols) ? 0 : c + 1;
            long long d = 0;
            for (int r = 0; r < rows; ++r) d += (long long)occ[r + rows * c] * occ[r + rows * cn];
            out[2 + rows + c] = d;
          }
        }
      } else if (lane == 0) {
        P.status[chain] = 1;  // sample buffer too small (host sizes it; never expected)
      }
      ++ns;
    }
  }
  __syncwarp();
  int8_t* gw = P.occ + (size_t)chain * N;
  for (int i = lane; i < N; i += 32) gw[i] = occ[i];
  for (int i = lane; i < MT_N; i += 32) gmt[i] = x[i];
  if (lane == 0) {
    gmt[MT_N] = (uint64_t)p;
    P.spin_sum[chain] = spin_sum;
    P.bond_sum[chain] = bond_sum;
    P.n_accept[chain] = n_acc;
    P.n_reject[chain] = n_rej;
    P.n_samples[chain] = ns;
  }
}

}  // namespace mg

// ---------------------------------------------------------------- C-ABI
struct mg_ising_replay {
  int rows = 0, cols = 0, n_chains = 0, use_nlist = 1;
  long long n_pass = 0;
  cudaStream_t stream = nullptr;
  double *dJ = nullptr, *dmu = nullptr, *dbeta = nullptr;
  int8_t* docc = nullptr;
  uint64_t* dmt = nullptr;
  long long *dspin = nullptr, *dbond = nullptr;
  unsigned long long *dacc = nullptr, *drej = nullptr;
  long long* dsamples = nullptr;
  int max_samples = 0;
  int *dns = nullptr, *dstatus = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
};

namespace {

void free_replay(mg_ising_replay* h) {
  if (!h) return;
  cudaFree(h->dJ);
  cudaFree(h->dmu);
  cudaFree(h->dbeta);
  cudaFree(h->docc);
  cudaFree(h->dmt);
  cudaFree(h->dspin);
  cudaFree(h->dbond);
  cudaFree(h->dacc);
  cudaFree(h->drej);
  cudaFree(h->dsamples);
  cudaFree(h->dns);
  cudaFree(h->dstatus);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

}  // namespace

extern "C" {

int mg_ising_replay_create(int rows, int cols, int n_chains, int use_nlist, const double* J,
                           const double* temperature, const double* mu, const int32_t* occ,
                           const char* const* engine_states, mg_ising_replay** out) {
  if (!out || rows < 1 || cols < 1 || n_chains < 1 || !J || !temperature || !mu || !occ ||
      !engine_states) {
    mg::set_error("Error in mg_ising_replay_create: invalid argument");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)rows * cols;
  if (N > 200000) {
    mg::set_error("Error in mg_ising_replay_create: supercell exceeds 200000 sites (shared-memory replay)");
    return MG_ERR_INVALID;
  }
  for (long long i = 0; i < N * n_chains; ++i) {
    if (occ[i] != 1 && occ[i] != -1) {
      mg::set_error("Error in mg_ising_replay_create: occupation values must be +1 or -1");
      return MG_ERR_INVALID;
    }
  }
  auto* h = new mg_ising_replay();
  h->rows = rows;
  h->cols = cols;
  h->n_chains = n_chains;
  h->use_nlist = use_nlist ? 1 : 0;
  std::vector<uint64_t> mt((size_t)n_chains * (mg::MT_N + 1));
  for (int c = 0; c < n_chains; ++c) {
    if (!engine_states[c] || mg::parse_mt_state(engine_states[c], mt.data() + (size_t)c * (mg::MT_N + 1))) {
      free_replay(h);
      mg::set_error("Error in mg_ising_replay_create: malformed engine state");
      return MG_ERR_INVALID;
    }
  }
  std::vector<double> beta(n_chains);
  const double KB = 8.6173303E-05;
  for (int c = 0; c < n_chains; ++c) beta[c] = 1.0 / (KB * temperature[c]);
  std::vector<int8_t> o8((size_t)N * n_chains);
  std::vector<long long> spin(n_chains, 0), bond(n_chains, 0);
  for (int c = 0; c < n_chains; ++c) {
    const int32_t* s = occ + (size_t)c * N;
    for (long long l = 0; l < N; ++l) o8[(size_t)c * N + l] = (int8_t)s[l];
    for (int j = 0; j < cols; ++j)
      for (int i = 0; i < rows; ++i) {
        const int l = i + rows * j;
        spin[c] += s[l];
        bond[c] += (long long)s[l] * (s[((i + 1) % rows) + rows * j] + s[i + rows * ((j + 1) % cols)]);
      }
  }
  auto fail = [&](cudaError_t e, const char* what) {
    mg::set_error(std::string("CUDA error in mg_ising_replay_create: ") + what + ": " + cudaGetErrorString(e));
    free_replay(h);
    return MG_ERR_CUDA;
  };
  cudaError_t e;
#define MGX(expr, what) \
  if ((e = (expr)) != cudaSuccess) return fail(e, what)
  MGX(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
  MGX(cudaMalloc(&h->dJ, sizeof(double) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dmu, sizeof(double) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dbeta, sizeof(double) * n_chains), "malloc");
  MGX(cudaMalloc(&h->docc, (size_t)N * n_chains), "malloc");
  MGX(cudaMalloc(&h->dmt, sizeof(uint64_t) * mt.size()), "malloc");
  MGX(cudaMalloc(&h->dspin, sizeof(long long) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dbond, sizeof(long long) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dacc, sizeof(unsigned long long) * n_chains), "malloc");
  MGX(cudaMalloc(&h->drej, sizeof(unsigned long long) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dns, sizeof(int) * n_chains), "malloc");
  MGX(cudaMalloc(&h->dstatus, sizeof(int) * n_chains), "malloc");
  MGX(cudaEventCreate(&h->ev0), "event");
  MGX(cudaEventCreate(&h->ev1), "event");
  MGX(cudaMemcpyAsync(h->dJ, J, sizeof(double) * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dmu, mu, sizeof(double) * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dbeta, beta.data(), sizeof(double) * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->docc, o8.data(), o8.size(), cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dmt, mt.data(), sizeof(uint64_t) * mt.size(), cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dspin, spin.data(), sizeof(long long) * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dbond, bond.data(), sizeof(long long) * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemsetAsync(h->dacc, 0, sizeof(unsigned long long) * n_chains, h->stream), "memset");
  MGX(cudaMemsetAsync(h->drej, 0, sizeof(unsigned long long) * n_chains, h->stream), "memset");
  MGX(cudaMemsetAsync(h->dstatus, 0, sizeof(int) * n_chains, h->stream), "memset");
  MGX(cudaStreamSynchronize(h->stream), "sync");
#undef MGX
  *out = h;
  return MG_OK;
}

int mg_ising_replay_run(mg_ising_replay* h, int n_passes, int sample_period,
                        long long* samples_out, int max_samples, int* n_samples_out) {
  if (!h || n_passes < 0 || sample_period < 1 || max_samples < 0 || (max_samples > 0 && !samples_out) ||
      !n_samples_out) {
    mg::set_error("Error in mg_ising_replay_run: invalid argument");
    return MG_ERR_INVALID;
  }
  const long long expected = (h->n_pass + n_passes) / sample_period - h->n_pass / sample_period;
  if (expected > max_samples) {
    mg::set_error("Error in mg_ising_replay_run: max_samples too small for the requested passes");
    return MG_ERR_INVALID;
  }
  const int stride = 2 + h->rows + h->cols;
  if (max_samples > h->max_samples) {
    cudaFree(h->dsamples);
    h->dsamples = nullptr;
    MG_CUDA_TRY(cudaMalloc(&h->dsamples, sizeof(long long) * (size_t)max_samples * stride * h->n_chains));
    h->max_samples = max_samples;
  }
  mg::IsingReplayParams P;
  P.rows = h->rows;
  P.cols = h->cols;
  P.n_chains = h->n_chains;
  P.use_nlist = h->use_nlist;
  P.sample_period = sample_period;
  P.pass0 = h->n_pass;
  P.n_passes = n_passes;
  P.max_samples = h->max_samples;
  P.J = h->dJ;
  P.mu = h->dmu;
  P.beta = h->dbeta;
  P.occ = h->docc;
  P.mt = h->dmt;
  P.spin_sum = h->dspin;
  P.bond_sum = h->dbond;
  P.n_accept = h->dacc;
  P.n_reject = h->drej;
  P.samples = h->dsamples;
  P.n_samples = h->dns;
  P.status = h->dstatus;
  const size_t smem = mg::MT_N * sizeof(uint64_t) + (size_t)h->rows * h->cols;
  if (smem > 48 * 1024) {
    MG_CUDA_TRY(cudaFuncSetAttribute(mg::ising_replay_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  MG_CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  mg::ising_replay_kernel<<<h->n_chains, 32, smem, h->stream>>>(P);
  MG_CUDA_TRY(cudaGetLastError());
  MG_CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
  std::vector<int> ns(h->n_chains), st(h->n_chains);
  MG_CUDA_TRY(cudaMemcpyAsync(ns.data(), h->dns, sizeof(int) * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(st.data(), h->dstatus, sizeof(int) * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  if (max_samples > 0) {
    // device rows are [chain][h->max_samples][stride]; the caller's are
    // [chain][max_samples][stride] with max_samples <= h->max_samples
    const size_t row = sizeof(long long) * (size_t)stride;
    MG_CUDA_TRY(cudaMemcpy2DAsync(samples_out, row * max_samples, h->dsamples, row * h->max_samples,
                                  row * max_samples, h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  }
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  for (int c = 0; c < h->n_chains; ++c) {
    if (st[c]) {
      mg::set_error("Error in mg_ising_replay_run: device reported a sample-buffer overflow");
      return MG_ERR_DEVICE;
    }
  }
  *n_samples_out = ns[0];
  h->n_pass += n_passes;
  return MG_OK;
}

int mg_ising_replay_get_state(mg_ising_replay* h, int32_t* occ, char** engine_states,
                              size_t state_len, unsigned long long* n_accept,
                              unsigned long long* n_reject) {
  if (!h) {
    mg::set_error("Error in mg_ising_replay_get_state: null handle");
    return MG_ERR_INVALID;
  }
  const size_t N = (size_t)h->rows * h->cols;
  std::vector<int8_t> o8(N * h->n_chains);
  std::vector<uint64_t> mt((size_t)h->n_chains * (mg::MT_N + 1));
  std::vector<unsigned long long> acc(h->n_chains), rej(h->n_chains);
  MG_CUDA_TRY(cudaMemcpyAsync(o8.data(), h->docc, o8.size(), cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(mt.data(), h->dmt, sizeof(uint64_t) * mt.size(), cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(acc.data(), h->dacc, sizeof(unsigned long long) * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(rej.data(), h->drej, sizeof(unsigned long long) * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (occ)
    for (size_t i = 0; i < o8.size(); ++i) occ[i] = o8[i];
  for (int c = 0; c < h->n_chains; ++c) {
    if (engine_states && engine_states[c]) {
      std::string s = mg::format_mt_state(mt.data() + (size_t)c * (mg::MT_N + 1));
      if (s.size() + 1 > state_len) {
        mg::set_error("Error in mg_ising_replay_get_state: engine state buffer too small");
        return MG_ERR_INVALID;
      }
      std::memcpy(engine_states[c], s.c_str(), s.size() + 1);
    }
    if (n_accept) n_accept[c] = acc[c];
    if (n_reject) n_reject[c] = rej[c];
  }
  return MG_OK;
}

int mg_ising_replay_last_kernel_ms(mg_ising_replay* h, float* ms) {
  if (!h || !ms) {
    mg::set_error("Error in mg_ising_replay_last_kernel_ms: invalid argument");
    return MG_ERR_INVALID;
  }
  *ms = h->last_ms;
  return MG_OK;
}

int mg_ising_replay_destroy(mg_ising_replay* h) {
  free_replay(h);
  return MG_OK;
}

}  // extern "C"

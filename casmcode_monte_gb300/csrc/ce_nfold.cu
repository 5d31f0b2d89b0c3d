// Host side and C-ABI of the rejection-free (N-fold way) sweep of ce_nfold.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/montegpu.h"
#include "ce_host.cuh"
#include "ce_nfold.cuh"
#include "mg_common.cuh"

struct mg_ce_nfold {
  const mg_ce_model* model = nullptr;
  int L0 = 0, L1 = 0, L2 = 0, n_chains = 0, n_super = 0;
  long long N = 0, events = 0;
  size_t smem = 0;
  bool small = false;  // the 128-thread instance
  mg::CeChainParams* dcp = nullptr;
  int8_t* docc = nullptr;
  long long* dcorr = nullptr;
  double* dout = nullptr;
  size_t out_cap = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
};

namespace {

using mg::set_error;
using namespace mg::host;

// Instances: 512 threads and one chain per SM; for supercells of at most kSmallSites sites,
// 128 threads and four chains per SM (at most 128 registers a thread, a quarter of the SM's
// shared memory each)
constexpr int kNtNfold = 512;
constexpr int kNtNfoldSmall = 128, kChainsPerSmSmall = 4, kSmallSites = 8192;

void free_nfold(mg_ce_nfold* h) {
  if (!h) return;
  cudaFree(h->dcp);
  cudaFree(h->docc);
  cudaFree(h->dcorr);
  cudaFree(h->dout);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// shared memory of one chain: rates and block sums of the padded site count, the lattice
// with its border
size_t nfold_smem(int L0, int L1, int L2, int n_super) {
  const size_t npad = (size_t)n_super * 1024;
  return sizeof(float) * (npad + npad / 32) +
         (size_t)(L0 + 2 * mg::CE_HALO) * (L1 + 2 * mg::CE_HALO) * (L2 + 2 * mg::CE_HALO);
}

int corr_recompute(mg_ce_nfold* h, long long* d) {
  MG_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(long long) * (size_t)h->model->n_classes * h->n_chains, h->stream));
  MG_CUDA_TRY(mg::host::launch_corr<mg::FccBinary>(h->docc, h->L0, h->L1, h->L2, h->n_chains, d, h->stream));
  return MG_OK;
}

}  // namespace

extern "C" {

int mg_ce_nfold_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains, const double* temperature,
                       const double* mu, const uint64_t* seeds, const uint32_t* chain_ids, const int8_t* occ,
                       mg_ce_nfold** out) {
  if (!m || !out || !temperature || !mu || !seeds || !occ || n_chains < 1) {
    set_error("Error in mg_ce_nfold_create: invalid argument");
    return MG_ERR_INVALID;
  }
  if (m->kind != 0) {
    set_error("Error in mg_ce_nfold_create: the rejection-free sweep flips sites of the binary basis");
    return MG_ERR_INVALID;
  }
  if (L0 < 4 || L1 < 4 || L2 < 4) {
    set_error("Error in mg_ce_nfold_create: supercell dimensions must be >= 4 (cluster images overlap)");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  if (N > mg::NFOLD_MAX_SITES) {
    set_error("Error in mg_ce_nfold_create: at most " + std::to_string(mg::NFOLD_MAX_SITES) +
              " sites per chain (the rates and their sums live in one CTA's shared memory)");
    return MG_ERR_INVALID;
  }
  for (long long i = 0; i < N * n_chains; ++i)
    if (occ[i] < 0 || occ[i] > 1) {
      set_error("Error in mg_ce_nfold_create: occupant index out of range");
      return MG_ERR_INVALID;
    }
  for (int c = 0; c < n_chains; ++c)
    if (!(temperature[c] > 0.0)) {
      set_error("Error in mg_ce_nfold_create: temperature must be > 0");
      return MG_ERR_INVALID;
    }
  const int n_super = (int)((N + 1023) / 1024);
  const size_t smem = nfold_smem(L0, L1, L2, n_super);
  int dev = 0, max_smem = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem + 2048 > (size_t)max_smem) {
    set_error("Error in mg_ce_nfold_create: the supercell's rates and lattice do not fit in one CTA's shared "
              "memory (" + std::to_string(smem) + " bytes)");
    return MG_ERR_INVALID;
  }
  auto* h = new mg_ce_nfold();
  h->model = m;
  h->L0 = L0;
  h->L1 = L1;
  h->L2 = L2;
  h->N = N;
  h->n_chains = n_chains;
  h->n_super = n_super;
  h->smem = smem;
  h->small = N <= kSmallSites && kChainsPerSmSmall * (smem + 1024) <= (size_t)max_smem;
  std::vector<mg::CeChainParams> cp(n_chains);
  make_chain_params(m, n_chains, temperature, mu, seeds, chain_ids, cp.data());
  auto fail = [&](cudaError_t e, const char* what) {
    set_error(std::string("CUDA error in mg_ce_nfold_create: ") + what + ": " + cudaGetErrorString(e));
    free_nfold(h);
    return MG_ERR_CUDA;
  };
  cudaError_t e;
#define MGX(expr, what) \
  if ((e = (expr)) != cudaSuccess) return fail(e, what)
  MGX(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
  MGX(cudaEventCreate(&h->ev0), "event");
  MGX(cudaEventCreate(&h->ev1), "event");
  MGX(cudaMalloc(&h->docc, (size_t)N * n_chains), "malloc occ");
  MGX(cudaMalloc(&h->dcp, sizeof(mg::CeChainParams) * n_chains), "malloc params");
  MGX(cudaMalloc(&h->dcorr, sizeof(long long) * (size_t)m->n_classes * n_chains), "malloc corr");
  MGX(cudaMemcpyAsync(h->docc, occ, (size_t)N * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dcp, cp.data(), sizeof(mg::CeChainParams) * n_chains, cudaMemcpyHostToDevice, h->stream),
      "copy");
#undef MGX
  const int rc = corr_recompute(h, h->dcorr);
  if (rc != MG_OK) {
    free_nfold(h);
    return rc;
  }
  if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return fail(e, "sync");
  *out = h;
  return MG_OK;
}

int mg_ce_nfold_run(mg_ce_nfold* h, int n_passes, double* out) {
  if (!h || n_passes < 0) {
    set_error("Error in mg_ce_nfold_run: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n_passes == 0) return MG_OK;
  const size_t nslot = (size_t)h->model->n_classes + 2;
  const size_t need = (size_t)n_passes * h->n_chains * nslot;
  if (need > h->out_cap) {
    cudaFree(h->dout);
    h->dout = nullptr;
    MG_CUDA_TRY(cudaMalloc(&h->dout, sizeof(double) * need));
    h->out_cap = need;
  }
  mg::CeNfoldArgs<mg::FccBinary::NFEAT> A;
  A.L0 = h->L0;
  A.L1 = h->L1;
  A.L2 = h->L2;
  A.PX = h->L0 + 2 * mg::CE_HALO;
  A.PY = h->L1 + 2 * mg::CE_HALO;
  A.n_super = h->n_super;
  fill_weights(h->model, A.w);
  A.cp = h->dcp;
  A.occ = h->docc;
  A.corr = h->dcorr;
  A.event0 = h->events;
  A.n_passes = n_passes;
  A.n_chains = h->n_chains;
  A.out = h->dout;
  int noff = 0;
  const int* off = offsets(0, &noff);
  if (noff != mg::NFOLD_NOFF) {
    set_error("Error in mg_ce_nfold_run: unexpected neighbour table");
    return MG_ERR_INVALID;
  }
  std::memcpy(A.offs, off, sizeof(int) * 3 * noff);
  auto kern = h->small ? mg::ce_nfold_kernel<mg::FccBinary, kNtNfoldSmall, kChainsPerSmSmall>
                       : mg::ce_nfold_kernel<mg::FccBinary, kNtNfold, 1>;
  const int nt = h->small ? kNtNfoldSmall : kNtNfold;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->smem));
  MG_CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  kern<<<h->n_chains, nt, h->smem, h->stream>>>(A);
  MG_CUDA_TRY(cudaGetLastError());
  MG_CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
  if (out) MG_CUDA_TRY(cudaMemcpyAsync(out, h->dout, sizeof(double) * need, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->events += (long long)n_passes * h->N;
  return MG_OK;
}

int mg_ce_nfold_info(const mg_ce_nfold* h, int* threads, int* chains_per_sm, size_t* smem_bytes) {
  if (!h) {
    set_error("Error in mg_ce_nfold_info: invalid argument");
    return MG_ERR_INVALID;
  }
  if (threads) *threads = h->small ? kNtNfoldSmall : kNtNfold;
  if (chains_per_sm) *chains_per_sm = h->small ? kChainsPerSmSmall : 1;
  if (smem_bytes) *smem_bytes = h->smem;
  return MG_OK;
}

int mg_ce_nfold_last_kernel_ms(const mg_ce_nfold* h, float* ms) {
  if (!h || !ms) {
    set_error("Error in mg_ce_nfold_last_kernel_ms: invalid argument");
    return MG_ERR_INVALID;
  }
  *ms = h->last_ms;
  return MG_OK;
}

int mg_ce_nfold_get_occ(mg_ce_nfold* h, int8_t* occ) {
  if (!h || !occ) {
    set_error("Error in mg_ce_nfold_get_occ: invalid argument");
    return MG_ERR_INVALID;
  }
  MG_CUDA_TRY(cudaMemcpyAsync(occ, h->docc, (size_t)h->N * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return MG_OK;
}

int mg_ce_nfold_corr(mg_ce_nfold* h, int recompute, long long* corr) {
  if (!h || !corr) {
    set_error("Error in mg_ce_nfold_corr: invalid argument");
    return MG_ERR_INVALID;
  }
  const size_t bytes = sizeof(long long) * (size_t)h->model->n_classes * h->n_chains;
  if (!recompute) {
    MG_CUDA_TRY(cudaMemcpyAsync(corr, h->dcorr, bytes, cudaMemcpyDeviceToHost, h->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return MG_OK;
  }
  long long* d = nullptr;
  MG_CUDA_TRY(cudaMalloc(&d, bytes));
  int rc = corr_recompute(h, d);
  cudaError_t e = cudaSuccess;
  if (rc == MG_OK) e = cudaMemcpyAsync(corr, d, bytes, cudaMemcpyDeviceToHost, h->stream);
  if (rc == MG_OK && e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (rc != MG_OK) return rc;
  if (e != cudaSuccess) {
    set_error(std::string("CUDA error in mg_ce_nfold_corr: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}

int mg_ce_nfold_destroy(mg_ce_nfold* h) {
  free_nfold(h);
  return MG_OK;
}

}  // extern "C"

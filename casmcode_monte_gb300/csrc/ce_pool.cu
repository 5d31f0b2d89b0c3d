// Chain pool: many independent cluster-expansion chains of any supercell shape resident
// in one HBM arena, swept by a persistent kernel (one CTA per chain, work queue ordered
// largest chain first).  Admission is by memory footprint: a chain is admitted only if
// its occupation fits in the arena (first-fit free list), which is what the serving
// loop uses to bound HBM use.  C-ABI in montegpu.h (mg_ce_pool_*).
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/montegpu.h"
#include "ce_host.cuh"
#include "mg_common.cuh"

namespace {

using mg::set_error;
using namespace mg::host;

constexpr int kMaxGeoms = 1024;

struct PoolGeom {
  int L0 = 0, L1 = 0, L2 = 0, n_colors = 0;
  int* dcstart = nullptr;
  uint32_t* dentries = nullptr;
  uint32_t* dsite = nullptr;
  std::vector<int32_t> color;
};

struct PoolSlot {
  bool used = false;
  int L0 = 0, L1 = 0, L2 = 0;
  long long N = 0, offset = 0, pass = 0;
  int geom = -1;
};

}  // namespace

struct mg_ce_pool {
  const mg_ce_model* model = nullptr;
  int precision = 0;
  long long arena_bytes = 0;
  int8_t* darena = nullptr;
  std::map<long long, long long> free_blocks;  // offset -> size
  std::vector<PoolSlot> slots;
  std::vector<PoolGeom> geoms;
  std::map<std::tuple<int, int, int>, int> geom_index;
  mg::CeChainParams* dcp = nullptr;
  mg::PoolGeometry* dgeoms = nullptr;
  mg::PoolItem* ditems = nullptr;
  int* dcounter = nullptr;
  long long* dcorr = nullptr;
  long long* dout = nullptr;
  size_t out_cap = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
};

namespace {

void free_pool(mg_ce_pool* p) {
  if (!p) return;
  for (auto& g : p->geoms) {
    cudaFree(g.dcstart);
    cudaFree(g.dentries);
    cudaFree(g.dsite);
  }
  cudaFree(p->darena);
  cudaFree(p->dcp);
  cudaFree(p->dgeoms);
  cudaFree(p->ditems);
  cudaFree(p->dcounter);
  cudaFree(p->dcorr);
  cudaFree(p->dout);
  if (p->ev0) cudaEventDestroy(p->ev0);
  if (p->ev1) cudaEventDestroy(p->ev1);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

bool arena_alloc(mg_ce_pool* p, long long n, long long* off) {
  const long long need = (n + 15) & ~15LL;
  for (auto it = p->free_blocks.begin(); it != p->free_blocks.end(); ++it) {
    if (it->second >= need) {
      *off = it->first;
      const long long rest = it->second - need;
      const long long roff = it->first + need;
      p->free_blocks.erase(it);
      if (rest > 0) p->free_blocks[roff] = rest;
      return true;
    }
  }
  return false;
}

void arena_free(mg_ce_pool* p, long long off, long long n) {
  const long long sz = (n + 15) & ~15LL;
  auto it = p->free_blocks.emplace(off, sz).first;
  auto next = std::next(it);
  if (next != p->free_blocks.end() && it->first + it->second == next->first) {
    it->second += next->second;
    p->free_blocks.erase(next);
  }
  if (it != p->free_blocks.begin()) {
    auto prev = std::prev(it);
    if (prev->first + prev->second == it->first) {
      prev->second += it->second;
      p->free_blocks.erase(it);
    }
  }
}

int geometry(mg_ce_pool* p, int L0, int L1, int L2, int* out) {
  auto key = std::make_tuple(L0, L1, L2);
  auto it = p->geom_index.find(key);
  if (it != p->geom_index.end()) {
    *out = it->second;
    return MG_OK;
  }
  if ((int)p->geoms.size() >= kMaxGeoms) {
    set_error("Error in mg_ce_pool_add: more than 1024 distinct supercell shapes");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  PoolGeom g;
  g.L0 = L0;
  g.L1 = L1;
  g.L2 = L2;
  g.color.assign(N, -1);
  g.n_colors = color_supercell(L0, L1, L2, p->model->kind, g.color.data());
  if (g.n_colors < 1) {
    set_error("Error in mg_ce_pool_add: colouring needs more than 64 colours");
    return MG_ERR_INVALID;
  }
  std::vector<int> cstart(g.n_colors + 1);
  std::vector<uint32_t> entries(N), site(N);
  build_site_lists(L0, L1, L2, 1, g.color.data(), g.n_colors, cstart.data(), entries.data(), site.data());
  MG_CUDA_TRY(cudaMalloc(&g.dcstart, sizeof(int) * cstart.size()));
  MG_CUDA_TRY(cudaMalloc(&g.dentries, sizeof(uint32_t) * N));
  MG_CUDA_TRY(cudaMalloc(&g.dsite, sizeof(uint32_t) * N));
  MG_CUDA_TRY(cudaMemcpyAsync(g.dcstart, cstart.data(), sizeof(int) * cstart.size(), cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(g.dentries, entries.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(g.dsite, site.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice, p->stream));
  mg::PoolGeometry dg{L0, L1, L2, g.n_colors, g.dcstart, g.dentries, g.dsite};
  const int gi = (int)p->geoms.size();
  MG_CUDA_TRY(cudaMemcpyAsync(p->dgeoms + gi, &dg, sizeof(dg), cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  p->geoms.push_back(std::move(g));
  p->geom_index[key] = gi;
  *out = gi;
  return MG_OK;
}

template <class B, int NT>
int launch_pool(mg_ce_pool* p, const std::vector<mg::PoolItem>& items, int n_passes, size_t smem) {
  mg::CePoolArgs<B::NFEAT> A;
  A.geoms = p->dgeoms;
  A.items = p->ditems;
  A.n_items = (int)items.size();
  A.next_item = p->dcounter;
  for (int k = 0; k < B::NFEAT; ++k) {
    A.w.w32[k] = p->model->w32[k];
    A.w.w64[k] = p->model->w64[k];
  }
  A.cp = p->dcp;
  A.occ = p->darena;
  A.n_passes = n_passes;
  A.precision = p->precision;
  A.out = p->dout;
  auto kern = mg::ce_pool_kernel<B, NT>;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, dev = 0, sms = 0;
  MG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem));
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (per_sm < 1) {
    set_error("Error in mg_ce_pool_run: the largest supercell does not fit in shared memory");
    return MG_ERR_INVALID;
  }
  const int grid = std::max(1, std::min((int)items.size(), per_sm * sms));
  kern<<<grid, NT, smem, p->stream>>>(A);
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

bool valid_slot(const mg_ce_pool* p, int slot) {
  return p && slot >= 0 && slot < (int)p->slots.size() && p->slots[slot].used;
}

}  // namespace

extern "C" {

int mg_ce_pool_create(const mg_ce_model* m, long long arena_bytes, int max_chains, int precision,
                      mg_ce_pool** out) {
  if (!m || !out || arena_bytes < 64 || max_chains < 1 || (precision != 0 && precision != 1)) {
    set_error("Error in mg_ce_pool_create: invalid argument");
    return MG_ERR_INVALID;
  }
  auto* p = new mg_ce_pool();
  p->model = m;
  p->precision = precision;
  p->arena_bytes = (arena_bytes + 15) & ~15LL;
  p->slots.resize(max_chains);
  p->free_blocks[0] = p->arena_bytes;
  cudaError_t e;
  auto fail = [&](const char* what) {
    set_error(std::string("CUDA error in mg_ce_pool_create: ") + what + ": " + cudaGetErrorString(e));
    free_pool(p);
    return MG_ERR_CUDA;
  };
  if ((e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream");
  if ((e = cudaEventCreate(&p->ev0)) != cudaSuccess) return fail("event");
  if ((e = cudaEventCreate(&p->ev1)) != cudaSuccess) return fail("event");
  if ((e = cudaMalloc(&p->darena, p->arena_bytes)) != cudaSuccess) return fail("arena");
  if ((e = cudaMalloc(&p->dcp, sizeof(mg::CeChainParams) * max_chains)) != cudaSuccess) return fail("params");
  if ((e = cudaMalloc(&p->dgeoms, sizeof(mg::PoolGeometry) * kMaxGeoms)) != cudaSuccess) return fail("geoms");
  if ((e = cudaMalloc(&p->ditems, sizeof(mg::PoolItem) * max_chains)) != cudaSuccess) return fail("items");
  if ((e = cudaMalloc(&p->dcounter, sizeof(int))) != cudaSuccess) return fail("counter");
  if ((e = cudaMalloc(&p->dcorr, sizeof(long long) * 64)) != cudaSuccess) return fail("corr");
  *out = p;
  return MG_OK;
}

int mg_ce_pool_add(mg_ce_pool* p, int L0, int L1, int L2, double temperature, const double* mu,
                   uint64_t seed, uint32_t chain_id, const int8_t* occ, int* slot_out) {
  if (!p || !occ || !slot_out || (p->model->n_species > 1 && !mu)) {
    set_error("Error in mg_ce_pool_add: invalid argument");
    return MG_ERR_INVALID;
  }
  if (L0 < 4 || L1 < 4 || L2 < 4) {
    set_error("Error in mg_ce_pool_add: supercell dimensions must be >= 4");
    return MG_ERR_INVALID;
  }
  if (!(temperature > 0.0)) {
    set_error("Error in mg_ce_pool_add: temperature must be > 0");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  for (long long i = 0; i < N; ++i)
    if (occ[i] < 0 || occ[i] >= p->model->n_species) {
      set_error("Error in mg_ce_pool_add: occupant index out of range");
      return MG_ERR_INVALID;
    }
  int dev = 0, max_smem = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (slab_smem(L0, L1, L2, 1) > (size_t)max_smem - 1024) {
    set_error("Error in mg_ce_pool_add: supercell does not fit in one CTA's shared memory (use a batch)");
    return MG_ERR_INVALID;
  }
  int slot = -1;
  for (int i = 0; i < (int)p->slots.size(); ++i)
    if (!p->slots[i].used) {
      slot = i;
      break;
    }
  if (slot < 0) {
    set_error("Error in mg_ce_pool_add: no free chain slot");
    return MG_ERR_FULL;
  }
  long long off = 0;
  if (!arena_alloc(p, N, &off)) {
    set_error("Error in mg_ce_pool_add: occupation does not fit in the arena");
    return MG_ERR_FULL;
  }
  int gi = -1;
  int rc = geometry(p, L0, L1, L2, &gi);
  if (rc != MG_OK) {
    arena_free(p, off, N);
    return rc;
  }
  mg::CeChainParams cp;
  make_chain_params(p->model, 1, &temperature, mu, &seed, &chain_id, &cp);
  MG_CUDA_TRY(cudaMemcpyAsync(p->darena + off, occ, N, cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(p->dcp + slot, &cp, sizeof(cp), cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  PoolSlot& s = p->slots[slot];
  s.used = true;
  s.L0 = L0;
  s.L1 = L1;
  s.L2 = L2;
  s.N = N;
  s.offset = off;
  s.pass = 0;
  s.geom = gi;
  *slot_out = slot;
  return MG_OK;
}

int mg_ce_pool_remove(mg_ce_pool* p, int slot) {
  if (!valid_slot(p, slot)) {
    set_error("Error in mg_ce_pool_remove: invalid slot");
    return MG_ERR_INVALID;
  }
  PoolSlot& s = p->slots[slot];
  arena_free(p, s.offset, s.N);
  s = PoolSlot();
  return MG_OK;
}

int mg_ce_pool_info(const mg_ce_pool* p, long long* arena_free_bytes, long long* arena_bytes, int* n_used,
                    int* max_chains) {
  if (!p) {
    set_error("Error in mg_ce_pool_info: null pool");
    return MG_ERR_INVALID;
  }
  long long fb = 0;
  for (auto& kv : p->free_blocks) fb += kv.second;
  int nu = 0;
  for (auto& s : p->slots) nu += s.used ? 1 : 0;
  if (arena_free_bytes) *arena_free_bytes = fb;
  if (arena_bytes) *arena_bytes = p->arena_bytes;
  if (n_used) *n_used = nu;
  if (max_chains) *max_chains = (int)p->slots.size();
  return MG_OK;
}

int mg_ce_pool_run(mg_ce_pool* p, const int32_t* slots, int n, int n_passes, long long* out) {
  if (!p || n < 0 || n_passes < 0 || (n > 0 && !slots)) {
    set_error("Error in mg_ce_pool_run: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n == 0 || n_passes == 0) return MG_OK;
  const int nslot = p->model->n_classes + 2;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) {
    if (!valid_slot(p, slots[i])) {
      set_error("Error in mg_ce_pool_run: invalid slot");
      return MG_ERR_INVALID;
    }
    order[i] = i;
  }
  // largest chains first (longest-processing-time order for the work queue)
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return p->slots[slots[a]].N > p->slots[slots[b]].N; });
  std::vector<mg::PoolItem> items(n);
  size_t smem = 0;
  for (int t = 0; t < n; ++t) {
    const int i = order[t];
    const PoolSlot& s = p->slots[slots[i]];
    items[t] = mg::PoolItem{s.geom, slots[i], s.offset, (long long)i * n_passes * nslot, s.pass};
    smem = std::max(smem, slab_smem(s.L0, s.L1, s.L2, 1));
  }
  const size_t need = (size_t)n * n_passes * nslot;
  if (need > p->out_cap) {
    cudaFree(p->dout);
    p->dout = nullptr;
    MG_CUDA_TRY(cudaMalloc(&p->dout, sizeof(long long) * need));
    p->out_cap = need;
  }
  if ((size_t)n > p->slots.size()) {
    set_error("Error in mg_ce_pool_run: more items than slots");
    return MG_ERR_INVALID;
  }
  MG_CUDA_TRY(cudaMemcpyAsync(p->ditems, items.data(), sizeof(mg::PoolItem) * n, cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaMemsetAsync(p->dcounter, 0, sizeof(int), p->stream));
  MG_CUDA_TRY(cudaEventRecord(p->ev0, p->stream));
  int rc = p->model->kind == 0 ? launch_pool<mg::FccBinary, mg::NT_BINARY>(p, items, n_passes, smem)
                               : launch_pool<mg::FccTernary, mg::NT_TERNARY>(p, items, n_passes, smem);
  if (rc != MG_OK) return rc;
  MG_CUDA_TRY(cudaEventRecord(p->ev1, p->stream));
  if (out) MG_CUDA_TRY(cudaMemcpyAsync(out, p->dout, sizeof(long long) * need, cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&p->last_ms, p->ev0, p->ev1));
  for (int i = 0; i < n; ++i) p->slots[slots[i]].pass += n_passes;
  return MG_OK;
}

int mg_ce_pool_last_kernel_ms(const mg_ce_pool* p, float* ms) {
  if (!p || !ms) {
    set_error("Error in mg_ce_pool_last_kernel_ms: invalid argument");
    return MG_ERR_INVALID;
  }
  *ms = p->last_ms;
  return MG_OK;
}

int mg_ce_pool_get_occ(mg_ce_pool* p, int slot, int8_t* occ) {
  if (!valid_slot(p, slot) || !occ) {
    set_error("Error in mg_ce_pool_get_occ: invalid argument");
    return MG_ERR_INVALID;
  }
  const PoolSlot& s = p->slots[slot];
  MG_CUDA_TRY(cudaMemcpyAsync(occ, p->darena + s.offset, s.N, cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return MG_OK;
}

int mg_ce_pool_colors(const mg_ce_pool* p, int slot, int32_t* color) {
  if (!valid_slot(p, slot) || !color) {
    set_error("Error in mg_ce_pool_colors: invalid argument");
    return MG_ERR_INVALID;
  }
  const PoolGeom& g = p->geoms[p->slots[slot].geom];
  std::copy(g.color.begin(), g.color.end(), color);
  return g.n_colors;
}

int mg_ce_pool_corr(mg_ce_pool* p, int slot, long long* out) {
  if (!valid_slot(p, slot) || !out) {
    set_error("Error in mg_ce_pool_corr: invalid argument");
    return MG_ERR_INVALID;
  }
  const PoolSlot& s = p->slots[slot];
  const int nc = p->model->n_classes;
  MG_CUDA_TRY(cudaMemsetAsync(p->dcorr, 0, sizeof(long long) * nc, p->stream));
  const int nblk = (int)std::min<long long>((s.N + 255) / 256, 1024);
  dim3 grid(nblk, 1);
  if (p->model->kind == 0)
    mg::ce_corr_kernel<mg::FccBinary><<<grid, 256, 0, p->stream>>>(p->darena + s.offset, s.L0, s.L1, s.L2, 1, p->dcorr);
  else
    mg::ce_corr_kernel<mg::FccTernary><<<grid, 256, 0, p->stream>>>(p->darena + s.offset, s.L0, s.L1, s.L2, 1, p->dcorr);
  MG_CUDA_TRY(cudaGetLastError());
  MG_CUDA_TRY(cudaMemcpyAsync(out, p->dcorr, sizeof(long long) * nc, cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return MG_OK;
}

int mg_ce_pool_destroy(mg_ce_pool* p) {
  free_pool(p);
  return MG_OK;
}

}  // extern "C"

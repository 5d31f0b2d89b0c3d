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
#include "stats.cuh"

namespace {

using mg::set_error;
using namespace mg::host;

constexpr int kMaxGeoms = 1024;
// CTA classes: chains are swept by 1, 2, 4, 8 or 16 CTAs (the smallest whose slab fits)
constexpr int kClasses = 5;
constexpr int kClassS[kClasses] = {1, 2, 4, 8, 16};
// launch groups: (CTA class, layout) with layout 0 = one site per byte, 1 = four per word,
// and the small byte-layout chains of class 1 whose padded lattice fits kWarpWindow bytes,
// swept one chain per warp (ce_pool_warp_kernel)
constexpr int kWarpGroup = 2 * kClasses;
// one-CTA word-layout chains of the binary basis whose lattice fits kSmallWindow bytes
// launch apart from the larger ones (a launch's shared memory is its largest chain's) with
// a kernel built for two CTAs per SM (80 registers), so that two such chains share an SM
constexpr int kSmallWordGroup = 2 * kClasses + 1;
constexpr int kGroups = 2 * kClasses + 2;
constexpr int kWarpWindow = 6144;
constexpr size_t kSmallWindow = 100 * 1024;
constexpr size_t kTwoPerSm = 110 * 1024;  // two CTAs' shared memory per SM (227 KB opt-in)
constexpr int kWarpsBinary = 16, kWarpsTernary = 12;

// bytes of a chain's padded byte-layout lattice, rounded to 16
inline int warp_window(int L0, int L1, int L2) {
  const long long w = (long long)(L0 + 2 * mg::CE_HALO) * (L1 + 2 * mg::CE_HALO) * (L2 + 2 * mg::CE_HALO);
  return (int)std::min<long long>((w + 15) & ~15LL, 1LL << 30);
}

struct PoolGeom {
  int L0 = 0, L1 = 0, L2 = 0, S = 1, layout = 0, n_colors = 0;
  int* dcstart = nullptr;
  uint32_t* dentries = nullptr;
  uint32_t* dsite = nullptr;
};

// per supercell shape: colouring, layout and CTA class (computed once)
struct ShapePlan {
  std::vector<int32_t> color;
  int n_colors = 0, layout = 0, cls = 0;
};

struct PoolSlot {
  bool used = false;
  int L0 = 0, L1 = 0, L2 = 0, cls = 0, layout = 0;
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
  std::map<std::tuple<int, int, int, int>, int> geom_index;
  std::map<std::tuple<int, int, int>, ShapePlan> plans;
  mg::CeChainParams* dcp = nullptr;
  mg::PoolGeometry* dgeoms = nullptr;
  mg::PoolItem* ditems = nullptr;
  int* dcounter = nullptr;  // one work counter per launch group
  long long* dcorr = nullptr;
  long long* dout = nullptr;
  size_t out_cap = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t cls_stream[kGroups] = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t cls_done[kGroups] = {};
  float last_ms = 0.f;
  int last_launches = 0;  // kernels launched by the last run
  // device-resident sample series (potential energy per site after every pass)
  int max_samples = 0;
  long long* dstate = nullptr;  // [slot][n_classes] integer correlation sums
  double* dseries = nullptr;    // [slot][max_samples]
  int* dnsamp = nullptr;        // [slot]
  double* dcheck = nullptr;     // check outputs
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
  cudaFree(p->dstate);
  cudaFree(p->dseries);
  cudaFree(p->dnsamp);
  cudaFree(p->dcheck);
  for (int c = 0; c < kGroups; ++c) {
    if (p->cls_stream[c]) cudaStreamDestroy(p->cls_stream[c]);
    if (p->cls_done[c]) cudaEventDestroy(p->cls_done[c]);
  }
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

// Colouring, layout and CTA class of a supercell shape (cached): the word layout where the
// basis and colouring allow it and some class fits it, else the byte layout; the class is
// the smallest CTA count whose slab fits in shared memory.
int shape_plan(mg_ce_pool* p, int L0, int L1, int L2, const ShapePlan** out) {
  auto key = std::make_tuple(L0, L1, L2);
  auto it = p->plans.find(key);
  if (it != p->plans.end()) {
    *out = &it->second;
    return MG_OK;
  }
  int dev = 0, max_smem = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  ShapePlan sp;
  sp.color.assign((size_t)L0 * L1 * L2, -1);
  sp.n_colors = color_supercell(L0, L1, L2, p->model->kind, sp.color.data());
  if (sp.n_colors < 1) {
    set_error("Error in mg_ce_pool_add: colouring needs more than 64 colours");
    return MG_ERR_INVALID;
  }
  auto fit = [&](int layout) {
    for (int c = 0; c < kClasses; ++c) {
      const int S = kClassS[c];
      if (slabs_ok(layout, L1, L2, S) && layout_smem(layout, L0, L1, L2, S) <= (size_t)max_smem - 1024) return c;
    }
    return -1;
  };
  sp.layout = 0;
  sp.cls = -1;
  if (quad_eligible(p->model->kind, L0, L1, L2, sp.color.data())) {
    sp.cls = fit(1);
    if (sp.cls >= 0) sp.layout = 1;
    // binary word chains too large for two one-CTA lattices per SM: a 2-CTA cluster whose
    // halves fit two per SM (kTwoPerSm) keeps twice the warps of one CTA per SM
    if (sp.cls == 0 && p->model->kind == 0 && layout_smem(1, L0, L1, L2, 1) > kSmallWindow && slabs_ok(1, L1, L2, 2) &&
        layout_smem(1, L0, L1, L2, 2) <= kTwoPerSm)
      sp.cls = 1;
  }
  if (sp.cls < 0) sp.cls = fit(0);
  if (sp.cls < 0) {
    set_error("Error in mg_ce_pool_add: supercell slab does not fit in shared memory with 16 CTAs");
    return MG_ERR_INVALID;
  }
  *out = &(p->plans[key] = std::move(sp));
  return MG_OK;
}

int geometry(mg_ce_pool* p, int L0, int L1, int L2, const ShapePlan& sp, int* out) {
  const int S = kClassS[sp.cls];
  auto key = std::make_tuple(L0, L1, L2, S);
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
  const long long n_entries = sp.layout == 1 ? N / 4 : N;
  PoolGeom g;
  g.L0 = L0;
  g.L1 = L1;
  g.L2 = L2;
  g.S = S;
  g.layout = sp.layout;
  g.n_colors = sp.n_colors;
  std::vector<int> cstart((size_t)S * (g.n_colors + 1));
  std::vector<uint32_t> entries(n_entries), site(n_entries);
  if (sp.layout == 1)
    build_word_lists(L0, L1, L2, S, sp.color.data(), g.n_colors, cstart.data(), entries.data(), site.data());
  else
    build_site_lists(L0, L1, L2, S, sp.color.data(), g.n_colors, p->model->kind, cstart.data(), entries.data(),
                     site.data());
  MG_CUDA_TRY(cudaMalloc(&g.dcstart, sizeof(int) * cstart.size()));
  MG_CUDA_TRY(cudaMalloc(&g.dentries, sizeof(uint32_t) * n_entries));
  MG_CUDA_TRY(cudaMalloc(&g.dsite, sizeof(uint32_t) * n_entries));
  MG_CUDA_TRY(cudaMemcpyAsync(g.dcstart, cstart.data(), sizeof(int) * cstart.size(), cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(g.dentries, entries.data(), sizeof(uint32_t) * n_entries, cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(g.dsite, site.data(), sizeof(uint32_t) * n_entries, cudaMemcpyHostToDevice, p->stream));
  const int planes = sp.layout == 1 ? word_slab_kind(L1, L2, S) : 1;
  mg::PoolGeometry dg{L0, L1, L2, g.n_colors, planes, g.dcstart, g.dentries, g.dsite};
  const int gi = (int)p->geoms.size();
  MG_CUDA_TRY(cudaMemcpyAsync(p->dgeoms + gi, &dg, sizeof(dg), cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  p->geoms.push_back(std::move(g));
  p->geom_index[key] = gi;
  *out = gi;
  return MG_OK;
}

// the word-layout pool kernel of basis B (binary: byte-parallel features; ternary: monomial
// counts, whose launch carries the count weights too)
template <class B, bool CLUSTER>
const void* pool_word_kernel(int* nt, bool two_per_sm = false) {
  if constexpr (B::NSPECIES == 3) {
    *nt = NT_TQUAD;
    return (const void*)mg::ce_pool_tquad_kernel<B, NT_TQUAD, CLUSTER>;
  } else {
    *nt = NT_QUAD;
    if (two_per_sm) return (const void*)mg::ce_pool_quad_kernel<B, NT_QUAD, CLUSTER, 2>;
    return (const void*)mg::ce_pool_quad_kernel<B, NT_QUAD, CLUSTER>;
  }
}

// the warp-per-chain kernel over the small byte-layout chains (win: the largest padded
// lattice of them, bytes)
template <class B>
int launch_pool_warp(mg_ce_pool* p, int item0, int n_items, int n_passes, int win) {
  constexpr int NW = B::NSPECIES == 3 ? kWarpsTernary : kWarpsBinary;
  mg::CePoolArgs<B::NFEAT> A;
  A.geoms = p->dgeoms;
  A.items = p->ditems + item0;
  A.n_items = n_items;
  A.next_item = p->dcounter + kWarpGroup;
  mg::host::fill_weights(p->model, A.w);
  A.cp = p->dcp;
  A.occ = p->darena;
  A.n_passes = n_passes;
  A.precision = p->precision;
  A.out = p->dout;
  const void* kern = (const void*)mg::ce_pool_warp_kernel<B, NW>;
  const size_t smem = (size_t)NW * win;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, dev = 0, sms = 0;
  MG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * NW, smem));
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (per_sm < 1) {
    set_error("Error in mg_ce_pool_run: the warp kernel does not fit on an SM");
    return MG_ERR_INVALID;
  }
  const int grid = std::max(1, std::min((n_items + NW - 1) / NW, per_sm * sms));
  void* args[] = {(void*)&A, (void*)&win};
  MG_CUDA_TRY(cudaLaunchKernel(kern, dim3(grid), dim3(32 * NW), args, smem, p->cls_stream[kWarpGroup]));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

template <class B, int NT>
int launch_pool(mg_ce_pool* p, int grp, int cls, int layout, int item0, int n_items, int n_passes, size_t smem) {
  mg::CeTPoolArgs<B::NFEAT, mg::FccTernary::NCOUNT> TA;  // the binary kernels read TA.p only
  mg::CePoolArgs<B::NFEAT>& A = TA.p;
  if constexpr (B::NSPECIES == 3) mg::host::fill_tquad_weights(p->model, TA.tw);
  A.geoms = p->dgeoms;
  A.items = p->ditems + item0;
  A.n_items = n_items;
  A.next_item = p->dcounter + grp;
  mg::host::fill_weights(p->model, A.w);
  A.cp = p->dcp;
  A.occ = p->darena;
  A.n_passes = n_passes;
  A.precision = p->precision;
  A.out = p->dout;
  const int S = kClassS[cls];
  cudaStream_t st = p->cls_stream[grp];
  if (S == 1) {
    const void* kern = (const void*)mg::ce_pool_kernel<B, NT>;
    int nt = NT;
    if (layout == 1) kern = pool_word_kernel<B, false>(&nt, grp == kSmallWordGroup);
    MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, dev = 0, sms = 0;
    MG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, smem));
    MG_CUDA_TRY(cudaGetDevice(&dev));
    MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (per_sm < 1) {
      set_error("Error in mg_ce_pool_run: supercell does not fit in shared memory");
      return MG_ERR_INVALID;
    }
    const int grid = std::max(1, std::min(n_items, per_sm * sms));
    void* args[] = {layout == 1 && B::NSPECIES == 3 ? (void*)&TA : (void*)&A};
    MG_CUDA_TRY(cudaLaunchKernel(kern, dim3(grid), dim3(nt), args, smem, st));
    MG_CUDA_TRY(cudaGetLastError());
    return MG_OK;
  }
  const void* kern = (const void*)mg::ce_pool_cluster_kernel<B, NT>;
  int nt = NT;
  if (layout == 1) kern = pool_word_kernel<B, true>(&nt, smem <= kTwoPerSm);
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (S > 8) MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(nt, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)S;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3((unsigned)S, 1, 1);
  int n_cl = 0;
  MG_CUDA_TRY(cudaOccupancyMaxActiveClusters(&n_cl, kern, &cfg));
  if (n_cl < 1) {
    set_error("Error in mg_ce_pool_run: no cluster of this size can be scheduled");
    return MG_ERR_INVALID;
  }
  cfg.gridDim = dim3((unsigned)(S * std::max(1, std::min(n_items, n_cl))), 1, 1);
  void* args[] = {layout == 1 && B::NSPECIES == 3 ? (void*)&TA : (void*)&A};
  MG_CUDA_TRY(cudaLaunchKernelExC(&cfg, kern, args));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

// Append one potential-energy-per-site sample per pass to each item's series: the
// item's integer correlation sums advance by the pass's changes; E_f = sum_f w_f C_f,
// E_pot = E_f - mu . N x, divided by N (same operation order as the host code).
template <int NC, int NSPEC>
__global__ void pool_series_kernel(const mg::PoolItem* items, int n_items, const mg::PoolGeometry* geoms,
                                   const mg::CeChainParams* cp, const long long* out, int n_passes,
                                   long long* state, double* series, int* nsamp, int max_samples,
                                   mg::CeWeightsClass<NC> wc) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const mg::PoolItem it = items[t];
  const mg::PoolGeometry g = geoms[it.geom];
  const long long N = (long long)g.L0 * g.L1 * g.L2;
  long long* C = state + (size_t)it.param * NC;
  double* ser = series + (size_t)it.param * max_samples;
  int ns = nsamp[it.param];
  const long long* o = out + it.out_offset;
  for (int p = 0; p < n_passes; ++p) {
    for (int f = 1; f < NC; ++f) C[f] += o[(size_t)p * (NC + 2) + f];
    double e = 0.0;
    for (int f = 0; f < NC; ++f) e = __dadd_rn(e, __dmul_rn(wc.w[f], (double)C[f]));
    double nx[2] = {0.0, 0.0};
    if (NSPEC == 2) {
      nx[0] = (double)C[1];
    } else {
      const long long nB = (N - C[2]) / 3;
      nx[0] = (double)nB;
      nx[1] = (double)((N - nB + C[1]) / 2);
    }
    for (int i = 0; i < NSPEC - 1; ++i) e = __dsub_rn(e, __dmul_rn(cp[it.param].mu[i], nx[i]));
    if (ns < max_samples) ser[ns] = __ddiv_rn(e, (double)N);
    ++ns;
  }
  nsamp[it.param] = ns;
}

// The reference's equilibration + convergence rule on one component per slot
// (EquilibrationCheck.cc:50-117, ConvergenceCheck.hh:74-184, BasicStatistics.cc:114-131):
// out[slot] = {equilibrated, N_equilibration, N_statistics, mean, precision, converged}.
__global__ void pool_check_kernel(const int* slots, int n, const double* series, const int* nsamp,
                                  int max_samples, double abs_precision, double confidence, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int slot = slots[t];
  const int N = min(nsamp[slot], max_samples);
  double* r = out + (size_t)t * 6;
  r[0] = 0.0;
  r[1] = 0.0;
  r[2] = 0.0;
  r[3] = 0.0;
  r[4] = DBL_MAX;
  r[5] = 0.0;
  if (N < 1) return;
  const double* x = series + (size_t)slot * max_samples;
  const mg::stats::Equilibration eq = mg::stats::equilibration_check(x, N, abs_precision);
  r[0] = eq.equilibrated ? 1.0 : 0.0;
  r[1] = (double)eq.n_equilibration;
  if (!eq.equilibrated || eq.n_equilibration >= N) return;
  const long n_stat = N - eq.n_equilibration;
  const mg::stats::MeanPrecision st = mg::stats::basic_statistics(x + eq.n_equilibration, n_stat, confidence);
  r[2] = (double)n_stat;
  r[3] = st.mean;
  r[4] = st.precision;
  r[5] = (st.precision < abs_precision) ? 1.0 : 0.0;
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
  for (int c = 0; c < kGroups; ++c) {
    if ((e = cudaStreamCreateWithFlags(&p->cls_stream[c], cudaStreamNonBlocking)) != cudaSuccess) return fail("stream");
    if ((e = cudaEventCreateWithFlags(&p->cls_done[c], cudaEventDisableTiming)) != cudaSuccess) return fail("event");
  }
  if ((e = cudaEventCreate(&p->ev0)) != cudaSuccess) return fail("event");
  if ((e = cudaEventCreate(&p->ev1)) != cudaSuccess) return fail("event");
  if ((e = cudaMalloc(&p->darena, p->arena_bytes)) != cudaSuccess) return fail("arena");
  if ((e = cudaMalloc(&p->dcp, sizeof(mg::CeChainParams) * max_chains)) != cudaSuccess) return fail("params");
  if ((e = cudaMalloc(&p->dgeoms, sizeof(mg::PoolGeometry) * kMaxGeoms)) != cudaSuccess) return fail("geoms");
  if ((e = cudaMalloc(&p->ditems, sizeof(mg::PoolItem) * max_chains)) != cudaSuccess) return fail("items");
  if ((e = cudaMalloc(&p->dcounter, sizeof(int) * kGroups)) != cudaSuccess) return fail("counter");
  if ((e = cudaMalloc(&p->dcorr, sizeof(long long) * 64)) != cudaSuccess) return fail("corr");
  *out = p;
  return MG_OK;
}

int mg_ce_pool_prepare(mg_ce_pool* p, int L0, int L1, int L2) {
  if (!p || L0 < 4 || L1 < 4 || L2 < 4) {
    set_error("Error in mg_ce_pool_prepare: invalid argument");
    return MG_ERR_INVALID;
  }
  const ShapePlan* sp = nullptr;
  int gi = 0;
  int rc = shape_plan(p, L0, L1, L2, &sp);
  if (rc != MG_OK) return rc;
  return geometry(p, L0, L1, L2, *sp, &gi);
}

namespace {

// the argument checks of one chain (dimensions, temperature, occupant codes)
int check_chain(const mg_ce_pool* p, const char* fn, int L0, int L1, int L2, double temperature,
                const int8_t* occ) {
  if (L0 < 4 || L1 < 4 || L2 < 4) {
    set_error(std::string("Error in ") + fn + ": supercell dimensions must be >= 4");
    return MG_ERR_INVALID;
  }
  if (!(temperature > 0.0)) {
    set_error(std::string("Error in ") + fn + ": temperature must be > 0");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  const int ns = p->model->n_species;
  int bad = 0;
  for (long long i = 0; i < N; ++i) bad |= (occ[i] < 0) | (occ[i] >= ns);
  if (bad) {
    set_error(std::string("Error in ") + fn + ": occupant index out of range");
    return MG_ERR_INVALID;
  }
  return MG_OK;
}

struct Reserved {
  int slot = -1, geom = -1;
  long long off = 0, N = 0;
  const ShapePlan* sp = nullptr;
};

// a free slot (searched from *hint on), arena space and the shape's geometry; the slot is
// marked used so that the next reservation skips it; on failure nothing is held
int reserve_chain(mg_ce_pool* p, const char* fn, int L0, int L1, int L2, int* hint, Reserved* r) {
  const int rc0 = shape_plan(p, L0, L1, L2, &r->sp);
  if (rc0 != MG_OK) return rc0;
  int slot = -1;
  for (int i = *hint; i < (int)p->slots.size(); ++i)
    if (!p->slots[i].used) {
      slot = i;
      break;
    }
  if (slot < 0) {
    set_error(std::string("Error in ") + fn + ": no free chain slot");
    return MG_ERR_FULL;
  }
  r->N = (long long)L0 * L1 * L2;
  if (!arena_alloc(p, r->N, &r->off)) {
    set_error(std::string("Error in ") + fn + ": occupation does not fit in the arena");
    return MG_ERR_FULL;
  }
  const int rc = geometry(p, L0, L1, L2, *r->sp, &r->geom);
  if (rc != MG_OK) {
    arena_free(p, r->off, r->N);
    return rc;
  }
  r->slot = slot;
  p->slots[slot].used = true;
  *hint = slot + 1;
  return MG_OK;
}

void release_chain(mg_ce_pool* p, const Reserved& r) {
  arena_free(p, r.off, r.N);
  p->slots[r.slot] = PoolSlot();
}

// the copies and series set-up of reserved chains (occupations from one host array, the
// chains' occupations back to back), merged where both sides are contiguous, then one
// stream synchronisation; fills the slot records
int admit_chains(mg_ce_pool* p, const Reserved* r, const int32_t* dims, int n, const int8_t* occ,
                 const mg::CeChainParams* cp) {
  long long src = 0;
  for (int i = 0; i < n;) {
    long long len = r[i].N, s0 = src, d0 = r[i].off;
    src += r[i].N;
    int j = i + 1;
    while (j < n && r[j].off == d0 + len && (r[j - 1].N & 15) == 0) {
      len += r[j].N;
      src += r[j].N;
      ++j;
    }
    MG_CUDA_TRY(cudaMemcpyAsync(p->darena + d0, occ + s0, (size_t)len, cudaMemcpyHostToDevice, p->stream));
    i = j;
  }
  for (int i = 0; i < n;) {
    int j = i + 1;
    while (j < n && r[j].slot == r[j - 1].slot + 1) ++j;
    MG_CUDA_TRY(cudaMemcpyAsync(p->dcp + r[i].slot, cp + i, sizeof(mg::CeChainParams) * (j - i),
                                cudaMemcpyHostToDevice, p->stream));
    i = j;
  }
  if (p->max_samples > 0) {
    // each series starts from the integer correlation sums of the initial occupation
    const int nc = p->model->n_classes;
    for (int i = 0; i < n; ++i) {
      long long* st = p->dstate + (size_t)r[i].slot * nc;
      MG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(long long) * nc, p->stream));
      MG_CUDA_TRY(cudaMemsetAsync(p->dnsamp + r[i].slot, 0, sizeof(int), p->stream));
      MG_CUDA_TRY(mg::host::launch_corr(p->model->kind, p->darena + r[i].off, dims[3 * i], dims[3 * i + 1],
                                        dims[3 * i + 2], 1, st, p->stream));
    }
  }
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  for (int i = 0; i < n; ++i) {
    PoolSlot& s = p->slots[r[i].slot];
    s.used = true;
    s.L0 = dims[3 * i];
    s.L1 = dims[3 * i + 1];
    s.L2 = dims[3 * i + 2];
    s.cls = r[i].sp->cls;
    s.layout = r[i].sp->layout;
    s.N = r[i].N;
    s.offset = r[i].off;
    s.pass = 0;
    s.geom = r[i].geom;
  }
  return MG_OK;
}

}  // namespace

int mg_ce_pool_add(mg_ce_pool* p, int L0, int L1, int L2, double temperature, const double* mu,
                   uint64_t seed, uint32_t chain_id, const int8_t* occ, int* slot_out) {
  if (!p || !occ || !slot_out || (p->model->n_species > 1 && !mu)) {
    set_error("Error in mg_ce_pool_add: invalid argument");
    return MG_ERR_INVALID;
  }
  const char* fn = "mg_ce_pool_add";
  int rc = check_chain(p, fn, L0, L1, L2, temperature, occ);
  if (rc != MG_OK) return rc;
  Reserved r;
  int hint = 0;
  rc = reserve_chain(p, fn, L0, L1, L2, &hint, &r);
  if (rc != MG_OK) return rc;
  mg::CeChainParams cp;
  make_chain_params(p->model, 1, &temperature, mu, &seed, &chain_id, &cp);
  const int32_t dims[3] = {L0, L1, L2};
  rc = admit_chains(p, &r, dims, 1, occ, &cp);
  if (rc != MG_OK) {
    release_chain(p, r);
    return rc;
  }
  *slot_out = r.slot;
  return MG_OK;
}

int mg_ce_pool_add_many(mg_ce_pool* p, int n, const int32_t* dims, const double* temperature, const double* mu,
                        const uint64_t* seeds, const uint32_t* chain_ids, const int8_t* occ, int32_t* slots_out) {
  if (!p || n < 0 || (n > 0 && (!dims || !temperature || !seeds || !chain_ids || !occ || !slots_out ||
                                (p->model->n_species > 1 && !mu)))) {
    set_error("Error in mg_ce_pool_add_many: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n == 0) return MG_OK;
  const char* fn = "mg_ce_pool_add_many";
  long long off = 0;
  for (int i = 0; i < n; ++i) {
    const int rc = check_chain(p, fn, dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], temperature[i], occ + off);
    if (rc != MG_OK) return rc;
    off += (long long)dims[3 * i] * dims[3 * i + 1] * dims[3 * i + 2];
  }
  std::vector<Reserved> r((size_t)n);
  int hint = 0;
  for (int i = 0; i < n; ++i) {
    const int rc = reserve_chain(p, fn, dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], &hint, &r[i]);
    if (rc != MG_OK) {
      for (int k = 0; k < i; ++k) release_chain(p, r[k]);
      return rc;
    }
  }
  std::vector<mg::CeChainParams> cp((size_t)n);
  make_chain_params(p->model, n, temperature, mu, seeds, chain_ids, cp.data());
  const int rc = admit_chains(p, r.data(), dims, n, occ, cp.data());
  if (rc != MG_OK) {
    for (int k = 0; k < n; ++k) release_chain(p, r[k]);
    return rc;
  }
  for (int i = 0; i < n; ++i) slots_out[i] = r[i].slot;
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
  if ((size_t)n > p->slots.size()) {
    set_error("Error in mg_ce_pool_run: more items than slots");
    return MG_ERR_INVALID;
  }
  const int nslot = p->model->n_classes + 2;
  std::vector<int> order(n);
  std::vector<char> seen(p->slots.size(), 0);
  for (int i = 0; i < n; ++i) {
    if (!valid_slot(p, slots[i]) || seen[slots[i]]) {
      set_error("Error in mg_ce_pool_run: invalid or repeated slot");
      return MG_ERR_INVALID;
    }
    seen[slots[i]] = 1;
    order[i] = i;
  }
  // grouped by launch group (CTA class, layout), largest chains first within a group
  // (LPT work queue)
  auto group = [&](const PoolSlot& x) {
    if (x.cls == 0 && x.layout == 0 && warp_window(x.L0, x.L1, x.L2) <= kWarpWindow) return kWarpGroup;
    if (p->model->kind == 0 && x.cls == 0 && x.layout == 1 && layout_smem(1, x.L0, x.L1, x.L2, 1) <= kSmallWindow)
      return kSmallWordGroup;
    return 2 * x.cls + x.layout;
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const PoolSlot &x = p->slots[slots[a]], &y = p->slots[slots[b]];
    if (group(x) != group(y)) return group(x) < group(y);
    return x.N > y.N;
  });
  std::vector<mg::PoolItem> items(n);
  int first[kGroups + 1] = {};
  size_t smem[kGroups] = {};
  for (int c = 0; c <= kGroups; ++c) first[c] = n;
  for (int t = n - 1; t >= 0; --t) {
    const int i = order[t];
    const PoolSlot& s = p->slots[slots[i]];
    items[t] = mg::PoolItem{s.geom, slots[i], s.offset, (long long)i * n_passes * nslot, s.pass};
    first[group(s)] = t;
    smem[group(s)] = std::max(smem[group(s)], group(s) == kWarpGroup
                                                  ? (size_t)warp_window(s.L0, s.L1, s.L2)
                                                  : layout_smem(s.layout, s.L0, s.L1, s.L2, kClassS[s.cls]));
  }
  for (int c = kGroups - 1; c >= 0; --c) first[c] = std::min(first[c], first[c + 1]);
  const size_t need = (size_t)n * n_passes * nslot;
  if (need > p->out_cap) {
    cudaFree(p->dout);
    p->dout = nullptr;
    MG_CUDA_TRY(cudaMalloc(&p->dout, sizeof(long long) * need));
    p->out_cap = need;
  }
  MG_CUDA_TRY(cudaMemcpyAsync(p->ditems, items.data(), sizeof(mg::PoolItem) * n, cudaMemcpyHostToDevice, p->stream));
  MG_CUDA_TRY(cudaMemsetAsync(p->dcounter, 0, sizeof(int) * kGroups, p->stream));
  MG_CUDA_TRY(cudaMemsetAsync(p->dout, 0, sizeof(long long) * need, p->stream));
  MG_CUDA_TRY(cudaEventRecord(p->ev0, p->stream));
  p->last_launches = 0;
  // one launch per group, each on its own stream after the set-up copies; the largest
  // class first so that its long chains start while the others fill in, the small-chain
  // groups last
  int launch_order[kGroups];
  for (int i = 0; i < 2 * kClasses; ++i) launch_order[i] = 2 * kClasses - 1 - i;
  launch_order[2 * kClasses] = kSmallWordGroup;
  launch_order[2 * kClasses + 1] = kWarpGroup;
  static_assert(kGroups == 2 * kClasses + 2, "the launch order covers every group");
  for (int oi = 0; oi < kGroups; ++oi) {
    const int c = launch_order[oi];
    const int cnt = first[c + 1] - first[c];
    if (cnt <= 0) continue;
    ++p->last_launches;
    MG_CUDA_TRY(cudaStreamWaitEvent(p->cls_stream[c], p->ev0, 0));
    const int cls = c == kSmallWordGroup ? 0 : c / 2, layout = c == kSmallWordGroup ? 1 : c % 2;
    int rc;
    if (c == kWarpGroup)
      rc = p->model->kind == 0 ? launch_pool_warp<mg::FccBinary>(p, first[c], cnt, n_passes, (int)smem[c])
                               : launch_pool_warp<mg::FccTernary>(p, first[c], cnt, n_passes, (int)smem[c]);
    else
      rc = p->model->kind == 0
               ? launch_pool<mg::FccBinary, mg::NT_BINARY>(p, c, cls, layout, first[c], cnt, n_passes, smem[c])
               : launch_pool<mg::FccTernary, mg::NT_TERNARY>(p, c, cls, layout, first[c], cnt, n_passes, smem[c]);
    if (rc != MG_OK) return rc;
    MG_CUDA_TRY(cudaEventRecord(p->cls_done[c], p->cls_stream[c]));
    MG_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->cls_done[c], 0));
  }
  MG_CUDA_TRY(cudaEventRecord(p->ev1, p->stream));
  if (p->max_samples > 0) {
    const int nc = p->model->n_classes;
    const int nt = 128, nb = (n + nt - 1) / nt;
    if (p->model->kind == 0) {
      mg::CeWeightsClass<mg::FccBinary::NCLASS> wc;
      for (int f = 0; f < nc; ++f) wc.w[f] = (p->model->eci[f] / (double)p->model->mult[f]) * p->model->scale[f];
      pool_series_kernel<mg::FccBinary::NCLASS, 2><<<nb, nt, 0, p->stream>>>(
          p->ditems, n, p->dgeoms, p->dcp, p->dout, n_passes, p->dstate, p->dseries, p->dnsamp, p->max_samples, wc);
    } else {
      mg::CeWeightsClass<mg::FccTernary::NCLASS> wc;
      for (int f = 0; f < nc; ++f) wc.w[f] = (p->model->eci[f] / (double)p->model->mult[f]) * p->model->scale[f];
      pool_series_kernel<mg::FccTernary::NCLASS, 3><<<nb, nt, 0, p->stream>>>(
          p->ditems, n, p->dgeoms, p->dcp, p->dout, n_passes, p->dstate, p->dseries, p->dnsamp, p->max_samples, wc);
    }
    MG_CUDA_TRY(cudaGetLastError());
    ++p->last_launches;
  }
  if (out) MG_CUDA_TRY(cudaMemcpyAsync(out, p->dout, sizeof(long long) * need, cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&p->last_ms, p->ev0, p->ev1));
  for (int i = 0; i < n; ++i) p->slots[slots[i]].pass += n_passes;
  return MG_OK;
}

int mg_ce_pool_enable_series(mg_ce_pool* p, int max_samples) {
  if (!p || max_samples < 1) {
    set_error("Error in mg_ce_pool_enable_series: invalid argument");
    return MG_ERR_INVALID;
  }
  for (auto& s : p->slots)
    if (s.used) {
      set_error("Error in mg_ce_pool_enable_series: enable before adding chains");
      return MG_ERR_INVALID;
    }
  const size_t nslots = p->slots.size();
  cudaFree(p->dstate);
  cudaFree(p->dseries);
  cudaFree(p->dnsamp);
  cudaFree(p->dcheck);
  p->dstate = nullptr;
  p->dseries = nullptr;
  p->dnsamp = nullptr;
  p->dcheck = nullptr;
  p->max_samples = 0;
  MG_CUDA_TRY(cudaMalloc(&p->dstate, sizeof(long long) * nslots * p->model->n_classes));
  MG_CUDA_TRY(cudaMalloc(&p->dseries, sizeof(double) * nslots * (size_t)max_samples));
  MG_CUDA_TRY(cudaMalloc(&p->dnsamp, sizeof(int) * nslots));
  MG_CUDA_TRY(cudaMalloc(&p->dcheck, sizeof(double) * 6 * nslots + sizeof(int) * nslots));
  MG_CUDA_TRY(cudaMemset(p->dnsamp, 0, sizeof(int) * nslots));
  p->max_samples = max_samples;
  return MG_OK;
}

int mg_ce_pool_series(mg_ce_pool* p, int slot, double* out, int max_n, int* n_out) {
  if (!valid_slot(p, slot) || !n_out || p->max_samples < 1 || (max_n > 0 && !out)) {
    set_error("Error in mg_ce_pool_series: invalid argument (series enabled?)");
    return MG_ERR_INVALID;
  }
  int ns = 0;
  MG_CUDA_TRY(cudaMemcpyAsync(&ns, p->dnsamp + slot, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  const int n = std::min(std::min(ns, p->max_samples), max_n);
  if (n > 0)
    MG_CUDA_TRY(cudaMemcpyAsync(out, p->dseries + (size_t)slot * p->max_samples, sizeof(double) * n,
                                cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  *n_out = ns;
  return MG_OK;
}

int mg_ce_pool_check(mg_ce_pool* p, const int32_t* slots, int n, double abs_precision, double confidence,
                     double* out) {
  if (!p || n < 0 || (n > 0 && (!slots || !out)) || p->max_samples < 1 || (size_t)n > p->slots.size()) {
    set_error("Error in mg_ce_pool_check: invalid argument (series enabled?)");
    return MG_ERR_INVALID;
  }
  if (n == 0) return MG_OK;
  for (int i = 0; i < n; ++i)
    if (!valid_slot(p, slots[i])) {
      set_error("Error in mg_ce_pool_check: invalid slot");
      return MG_ERR_INVALID;
    }
  double* dres = p->dcheck;
  int* dslots = reinterpret_cast<int*>(p->dcheck + 6 * p->slots.size());
  MG_CUDA_TRY(cudaMemcpyAsync(dslots, slots, sizeof(int) * n, cudaMemcpyHostToDevice, p->stream));
  const int nt = 32, nb = (n + nt - 1) / nt;
  pool_check_kernel<<<nb, nt, 0, p->stream>>>(dslots, n, p->dseries, p->dnsamp, p->max_samples, abs_precision,
                                               confidence, dres);
  MG_CUDA_TRY(cudaGetLastError());
  MG_CUDA_TRY(cudaMemcpyAsync(out, dres, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
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

int mg_ce_pool_last_launches(const mg_ce_pool* p, int* n) {
  if (!p || !n) {
    set_error("Error in mg_ce_pool_last_launches: invalid argument");
    return MG_ERR_INVALID;
  }
  *n = p->last_launches;
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
  const PoolSlot& sl = p->slots[slot];
  const ShapePlan& sp = p->plans.at(std::make_tuple(sl.L0, sl.L1, sl.L2));
  std::copy(sp.color.begin(), sp.color.end(), color);
  return sp.n_colors;
}

int mg_ce_pool_corr(mg_ce_pool* p, int slot, long long* out) {
  if (!valid_slot(p, slot) || !out) {
    set_error("Error in mg_ce_pool_corr: invalid argument");
    return MG_ERR_INVALID;
  }
  const PoolSlot& s = p->slots[slot];
  const int nc = p->model->n_classes;
  MG_CUDA_TRY(cudaMemsetAsync(p->dcorr, 0, sizeof(long long) * nc, p->stream));
  MG_CUDA_TRY(mg::host::launch_corr(p->model->kind, p->darena + s.offset, s.L0, s.L1, s.L2, 1, p->dcorr, p->stream));
  MG_CUDA_TRY(cudaMemcpyAsync(out, p->dcorr, sizeof(long long) * nc, cudaMemcpyDeviceToHost, p->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return MG_OK;
}

int mg_ce_pool_destroy(mg_ce_pool* p) {
  free_pool(p);
  return MG_OK;
}

}  // extern "C"

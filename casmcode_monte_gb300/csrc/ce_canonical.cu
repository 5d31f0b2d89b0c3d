// Host side and C-ABI of the canonical (fixed-composition) sweep of ce_canonical.cuh:
// the two colourings, their per-colour site lists, chain parameters and the kernel dispatch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/montegpu.h"
#include "ce_canonical.cuh"
#include "ce_host.cuh"
#include "mg_common.cuh"

struct mg_ce_canon {
  const mg_ce_model* model = nullptr;
  int L0 = 0, L1 = 0, L2 = 0, n_chains = 0, precision = 0;
  long long N = 0;
  int PX = 0, PY = 0, threads = 0;
  size_t smem = 0;
  int n_colors[2] = {0, 0};
  std::vector<int32_t> color[2];
  std::vector<int32_t> order[2];  // list sites of each colouring, colour by colour
  int* dcstart[2] = {nullptr, nullptr};
  uint32_t* dentries[2] = {nullptr, nullptr};
  uint32_t* dsite[2] = {nullptr, nullptr};
  mg::CeChainParams* dcp = nullptr;
  int8_t* docc = nullptr;
  long long* dout = nullptr;
  size_t out_cap = 0;
  long long pass = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
};

namespace {

using mg::set_error;
using namespace mg::host;

// threads per CTA of the ternary canonical kernel: two sites' features per thread need up
// to 255 registers (no spills); the binary kernel runs NT_BINARY threads
constexpr int kNtCanonTernary = 256;

void free_canon(mg_ce_canon* h) {
  if (!h) return;
  for (int t = 0; t < 2; ++t) {
    cudaFree(h->dcstart[t]);
    cudaFree(h->dentries[t]);
    cudaFree(h->dsite[t]);
  }
  cudaFree(h->dcp);
  cudaFree(h->docc);
  cudaFree(h->dout);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// True when the classes of colourings a and b join into one connected set: class alpha of a
// and class beta of b are linked when some site has both; union-find over the classes.
bool colourings_connected(const int32_t* a, int na, const int32_t* b, int nb, long long N) {
  std::vector<int> parent(na + nb);
  std::iota(parent.begin(), parent.end(), 0);
  auto find = [&](int x) {
    while (parent[x] != x) x = parent[x] = parent[parent[x]];
    return x;
  };
  std::vector<char> used(na + nb, 0);
  for (long long l = 0; l < N; ++l) {
    const int x = find(a[l]), y = find(na + b[l]);
    used[a[l]] = used[na + b[l]] = 1;
    if (x != y) parent[x] = y;
  }
  int root = -1;
  for (int c = 0; c < na + nb; ++c) {
    if (!used[c]) continue;
    const int r = find(c);
    if (root < 0) root = r;
    if (r != root) return false;
  }
  return true;
}

// (a i + b j + c k) mod m is a valid colouring of the supercell's conflict graph (periodic,
// and no cluster offset maps to colour 0)
bool linear_valid(int kind, int L0, int L1, int L2, int a, int b, int c, int m) {
  if ((1LL * a * L0) % m || (1LL * b * L1) % m || (1LL * c * L2) % m) return false;
  int noff = 0;
  const int* off = offsets(kind, &noff);
  for (int t = 0; t < noff; ++t) {
    long long v = (1LL * a * off[3 * t] + 1LL * b * off[3 * t + 1] + 1LL * c * off[3 * t + 2]) % m;
    if (v < 0) v += m;
    if (v == 0) return false;
  }
  return true;
}

// Greedy colouring visiting the sites in the given order: another valid colouring for
// supercells without a second linear one.
int greedy_in_order(int kind, int L0, int L1, int L2, const std::vector<long long>& order, int32_t* col) {
  int noff = 0;
  const int* off = offsets(kind, &noff);
  const long long N = (long long)L0 * L1 * L2;
  std::fill(col, col + N, -1);
  int n_colors = 0;
  for (const long long l : order) {
    const int i = (int)(l % L0), j = (int)((l / L0) % L1), k = (int)(l / ((long long)L0 * L1));
    unsigned long long used = 0ull;
    for (int t = 0; t < noff; ++t) {
      const int a = ((i + off[3 * t]) % L0 + L0) % L0, b = ((j + off[3 * t + 1]) % L1 + L1) % L1,
                c = ((k + off[3 * t + 2]) % L2 + L2) % L2;
      const int32_t cc = col[a + (long long)L0 * (b + (long long)L1 * c)];
      if (cc >= 0) used |= 1ull << cc;
    }
    if (used == ~0ull) return -1;
    int cc = 0;
    while (used >> cc & 1ull) ++cc;
    col[l] = cc;
    n_colors = std::max(n_colors, cc + 1);
  }
  return n_colors;
}

// The two colourings of the canonical sweep: A is the sweep's own colouring
// (color_supercell); B the first valid linear colouring (by modulus, then coefficients)
// whose classes join A's into one connected set, else the first greedy colouring that
// connects (reverse site order, then up to 15 shuffled orders).  False when none connects.
bool canonical_colourings(int kind, int L0, int L1, int L2, mg_ce_canon* h) {
  const long long N = (long long)L0 * L1 * L2;
  h->color[0].assign(N, 0);
  h->color[1].assign(N, 0);
  h->n_colors[0] = color_supercell(L0, L1, L2, kind, h->color[0].data());
  if (h->n_colors[0] < 1) return false;
  for (int m = 2; m <= 32; ++m)
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b)
        for (int c = 0; c < m; ++c) {
          if (!linear_valid(kind, L0, L1, L2, a, b, c, m)) continue;
          for (int k = 0; k < L2; ++k)
            for (int j = 0; j < L1; ++j)
              for (int i = 0; i < L0; ++i)
                h->color[1][i + (long long)L0 * (j + (long long)L1 * k)] =
                    (int32_t)((1LL * a * i + 1LL * b * j + 1LL * c * k) % m);
          if (colourings_connected(h->color[0].data(), h->n_colors[0], h->color[1].data(), m, N)) {
            h->n_colors[1] = m;
            return true;
          }
        }
  // greedy colourings: reverse site order, then site orders shuffled by a fixed generator
  // (splitmix64 and Fisher-Yates: the same orders on every platform)
  std::vector<long long> order(N);
  for (long long l = 0; l < N; ++l) order[l] = N - 1 - l;
  uint64_t z = 0x9E3779B97F4A7C15ull;
  auto next = [&]() {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
  };
  for (int attempt = 0; attempt < 16; ++attempt) {
    if (attempt > 0)
      for (long long l = N - 1; l > 0; --l) std::swap(order[l], order[(long long)(next() % (uint64_t)(l + 1))]);
    h->n_colors[1] = greedy_in_order(kind, L0, L1, L2, order, h->color[1].data());
    if (h->n_colors[1] >= 1 &&
        colourings_connected(h->color[0].data(), h->n_colors[0], h->color[1].data(), h->n_colors[1], N))
      return true;
  }
  return false;
}

// Per-colour lists of one colouring for one CTA holding the whole lattice: entry = padded
// index | flags << 24 (flags: the site's periodic copies, as SiteSweeper::store reads them),
// site = linear index.  Within a colour the sites are ordered for shared-memory banks, as the
// sweep's byte lists are: by residue g = padded index & 3, then round-robin over the 32 banks
// (bank q = (padded index >> 2) & 31): the first site of every bank, then the second, ... (in
// ascending site order within a bank), so that consecutive list positions, which adjacent
// lanes take, fall in different banks.  The matching pairs list positions, so the order is
// part of the trajectory (mg_ce_canon_class_order returns it).
void canonical_lists(int L0, int L1, int L2, const int32_t* col, int nc, std::vector<int>& cstart,
                     std::vector<uint32_t>& entries, std::vector<uint32_t>& site) {
  const long long N = (long long)L0 * L1 * L2;
  const int H = mg::CE_HALO;
  const int PX = L0 + 2 * H, PY = L1 + 2 * H;
  std::vector<std::vector<std::vector<long long>>> bucket((size_t)nc, std::vector<std::vector<long long>>(128));
  std::vector<uint32_t> pidx_of(N);
  for (long long l = 0; l < N; ++l) {
    const int i = (int)(l % L0), j = (int)((l / L0) % L1), k = (int)(l / ((long long)L0 * L1));
    const uint32_t pidx = (uint32_t)((i + H) + PX * ((j + H) + PY * (k + H)));
    pidx_of[l] = pidx;
    bucket[col[l]][(pidx & 3u) * 32u + ((pidx >> 2) & 31u)].push_back(l);
  }
  cstart.assign(nc + 1, 0);
  entries.assign(N, 0u);
  site.assign(N, 0u);
  long long p = 0;
  for (int c = 0; c < nc; ++c) {
    cstart[c] = (int)p;
    for (int g = 0; g < 4; ++g) {
      size_t rounds = 0;
      for (int q = 0; q < 32; ++q) rounds = std::max(rounds, bucket[c][g * 32 + q].size());
      for (size_t t = 0; t < rounds; ++t)
        for (int q = 0; q < 32; ++q) {
          const auto& b = bucket[c][g * 32 + q];
          if (t >= b.size()) continue;
          const long long l = b[t];
          const int i = (int)(l % L0), j = (int)((l / L0) % L1), k = (int)(l / ((long long)L0 * L1));
          uint32_t flags = 0;
          if (i < H) flags |= 1;
          else if (i >= L0 - H) flags |= 2;
          if (j < H) flags |= 4;
          else if (j >= L1 - H) flags |= 8;
          if (k < H) flags |= 16;
          if (k >= L2 - H) flags |= 32;
          entries[p] = pidx_of[l] | (flags << 24);
          site[p] = (uint32_t)l;
          ++p;
        }
    }
  }
  cstart[nc] = (int)p;
}

template <class B, int NT>
int launch_canonical_t(const mg_ce_canon* h, int n_passes) {
  mg::CeCanonArgs<B::NFEAT> A;
  A.L0 = h->L0;
  A.L1 = h->L1;
  A.L2 = h->L2;
  A.PX = h->PX;
  A.PY = h->PY;
  for (int t = 0; t < 2; ++t) {
    A.col[t].n_colors = h->n_colors[t];
    A.col[t].color_start = h->dcstart[t];
    A.col[t].entries = h->dentries[t];
    A.col[t].site_l = h->dsite[t];
  }
  fill_weights(h->model, A.w);
  A.cp = h->dcp;
  A.occ = h->docc;
  A.pass0 = h->pass;
  A.n_passes = n_passes;
  A.n_chains = h->n_chains;
  A.precision = h->precision;
  A.out = h->dout;
  auto kern = mg::ce_canonical_kernel<B, NT>;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->smem));
  kern<<<h->n_chains, NT, h->smem, h->stream>>>(A);
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

}  // namespace

extern "C" {

int mg_ce_canon_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains, const double* temperature,
                       const uint64_t* seeds, const uint32_t* chain_ids, const int8_t* occ, int precision,
                       mg_ce_canon** out) {
  if (!m || !out || !temperature || !seeds || !occ || n_chains < 1) {
    set_error("Error in mg_ce_canon_create: invalid argument");
    return MG_ERR_INVALID;
  }
  if (L0 < 4 || L1 < 4 || L2 < 4) {
    set_error("Error in mg_ce_canon_create: supercell dimensions must be >= 4 (cluster images overlap)");
    return MG_ERR_INVALID;
  }
  if (precision != 0 && precision != 1) {
    set_error("Error in mg_ce_canon_create: precision must be 0 (FP64) or 1 (FP32)");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  const size_t smem = (size_t)(L0 + 2 * mg::CE_HALO) * (L1 + 2 * mg::CE_HALO) * (L2 + 2 * mg::CE_HALO);
  int dev = 0, max_smem = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem + 1024 > (size_t)max_smem) {
    set_error("Error in mg_ce_canon_create: the supercell with its border does not fit in one CTA's shared "
              "memory (" + std::to_string(smem) + " bytes)");
    return MG_ERR_INVALID;
  }
  for (long long i = 0; i < N * n_chains; ++i)
    if (occ[i] < 0 || occ[i] >= m->n_species) {
      set_error("Error in mg_ce_canon_create: occupant index out of range");
      return MG_ERR_INVALID;
    }
  for (int c = 0; c < n_chains; ++c)
    if (!(temperature[c] > 0.0)) {
      set_error("Error in mg_ce_canon_create: temperature must be > 0");
      return MG_ERR_INVALID;
    }
  auto* h = new mg_ce_canon();
  h->model = m;
  h->L0 = L0;
  h->L1 = L1;
  h->L2 = L2;
  h->N = N;
  h->n_chains = n_chains;
  h->precision = precision;
  h->PX = L0 + 2 * mg::CE_HALO;
  h->PY = L1 + 2 * mg::CE_HALO;
  h->smem = smem;
  h->threads = m->kind == 0 ? mg::NT_BINARY : kNtCanonTernary;
  if (!canonical_colourings(m->kind, L0, L1, L2, h)) {
    delete h;
    set_error("Error in mg_ce_canon_create: no pair of colourings of this supercell connects its sites");
    return MG_ERR_INVALID;
  }
  // chain parameters: no exchange potential; the decision bounds of a swap are those of two
  // flips (twice the quantisation error and twice the largest energy change)
  mg_ce_model m2 = *m;
  m2.qerr = 2.0 * m->qerr;
  m2.qmax = 2.0 * m->qmax;
  std::vector<double> mu((size_t)n_chains * (m->n_species - 1), 0.0);
  std::vector<mg::CeChainParams> cp(n_chains);
  make_chain_params(&m2, n_chains, temperature, mu.data(), seeds, chain_ids, cp.data());

  auto fail = [&](cudaError_t e, const char* what) {
    set_error(std::string("CUDA error in mg_ce_canon_create: ") + what + ": " + cudaGetErrorString(e));
    free_canon(h);
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
  MGX(cudaMemcpyAsync(h->docc, occ, (size_t)N * n_chains, cudaMemcpyHostToDevice, h->stream), "copy");
  MGX(cudaMemcpyAsync(h->dcp, cp.data(), sizeof(mg::CeChainParams) * n_chains, cudaMemcpyHostToDevice, h->stream),
      "copy");
  for (int t = 0; t < 2; ++t) {
    std::vector<int> cstart;
    std::vector<uint32_t> entries, site;
    canonical_lists(L0, L1, L2, h->color[t].data(), h->n_colors[t], cstart, entries, site);
    h->order[t].assign(site.begin(), site.end());
    MGX(cudaMalloc(&h->dcstart[t], sizeof(int) * cstart.size()), "malloc lists");
    MGX(cudaMalloc(&h->dentries[t], sizeof(uint32_t) * entries.size()), "malloc lists");
    MGX(cudaMalloc(&h->dsite[t], sizeof(uint32_t) * site.size()), "malloc lists");
    MGX(cudaMemcpyAsync(h->dcstart[t], cstart.data(), sizeof(int) * cstart.size(), cudaMemcpyHostToDevice, h->stream),
        "copy");
    MGX(cudaMemcpyAsync(h->dentries[t], entries.data(), sizeof(uint32_t) * entries.size(), cudaMemcpyHostToDevice,
                        h->stream),
        "copy");
    MGX(cudaMemcpyAsync(h->dsite[t], site.data(), sizeof(uint32_t) * site.size(), cudaMemcpyHostToDevice, h->stream),
        "copy");
    MGX(cudaStreamSynchronize(h->stream), "sync");  // the host lists go out of scope
  }
#undef MGX
  *out = h;
  return MG_OK;
}

int mg_ce_canon_info(const mg_ce_canon* h, int* n_colors_a, int* n_colors_b, int* threads, size_t* smem_bytes) {
  if (!h) {
    set_error("Error in mg_ce_canon_info: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n_colors_a) *n_colors_a = h->n_colors[0];
  if (n_colors_b) *n_colors_b = h->n_colors[1];
  if (threads) *threads = h->threads;
  if (smem_bytes) *smem_bytes = h->smem;
  return MG_OK;
}

int mg_ce_canon_colors(const mg_ce_canon* h, int which, int32_t* color) {
  if (!h || !color || which < 0 || which > 1) {
    set_error("Error in mg_ce_canon_colors: invalid argument");
    return MG_ERR_INVALID;
  }
  std::memcpy(color, h->color[which].data(), sizeof(int32_t) * (size_t)h->N);
  return MG_OK;
}

int mg_ce_canon_class_order(const mg_ce_canon* h, int which, int32_t* site_order) {
  if (!h || !site_order || which < 0 || which > 1) {
    set_error("Error in mg_ce_canon_class_order: invalid argument");
    return MG_ERR_INVALID;
  }
  std::memcpy(site_order, h->order[which].data(), sizeof(int32_t) * (size_t)h->N);
  return MG_OK;
}

int mg_ce_canon_run(mg_ce_canon* h, int n_passes, long long* out) {
  if (!h || n_passes < 0) {
    set_error("Error in mg_ce_canon_run: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n_passes == 0) return MG_OK;
  const size_t nslot = (size_t)h->model->n_classes + 2;
  const size_t need = (size_t)n_passes * h->n_chains * nslot;
  if (need > h->out_cap) {
    cudaFree(h->dout);
    h->dout = nullptr;
    MG_CUDA_TRY(cudaMalloc(&h->dout, sizeof(long long) * need));
    h->out_cap = need;
  }
  MG_CUDA_TRY(cudaMemsetAsync(h->dout, 0, sizeof(long long) * need, h->stream));
  MG_CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  const int rc = h->model->kind == 0 ? launch_canonical_t<mg::FccBinary, mg::NT_BINARY>(h, n_passes)
                                     : launch_canonical_t<mg::FccTernary, kNtCanonTernary>(h, n_passes);
  if (rc != MG_OK) return rc;
  MG_CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
  if (out) MG_CUDA_TRY(cudaMemcpyAsync(out, h->dout, sizeof(long long) * need, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->pass += n_passes;
  return MG_OK;
}

int mg_ce_canon_last_kernel_ms(const mg_ce_canon* h, float* ms) {
  if (!h || !ms) {
    set_error("Error in mg_ce_canon_last_kernel_ms: invalid argument");
    return MG_ERR_INVALID;
  }
  *ms = h->last_ms;
  return MG_OK;
}

int mg_ce_canon_get_occ(mg_ce_canon* h, int8_t* occ) {
  if (!h || !occ) {
    set_error("Error in mg_ce_canon_get_occ: invalid argument");
    return MG_ERR_INVALID;
  }
  MG_CUDA_TRY(cudaMemcpyAsync(occ, h->docc, (size_t)h->N * h->n_chains, cudaMemcpyDeviceToHost, h->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return MG_OK;
}

int mg_ce_canon_corr(mg_ce_canon* h, long long* out) {
  if (!h || !out) {
    set_error("Error in mg_ce_canon_corr: invalid argument");
    return MG_ERR_INVALID;
  }
  const int nc = h->model->n_classes;
  long long* d = nullptr;
  MG_CUDA_TRY(cudaMalloc(&d, sizeof(long long) * (size_t)nc * h->n_chains));
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(long long) * (size_t)nc * h->n_chains, h->stream);
  if (e == cudaSuccess) e = mg::host::launch_corr(h->model->kind, h->docc, h->L0, h->L1, h->L2, h->n_chains, d, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d, sizeof(long long) * (size_t)nc * h->n_chains, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error(std::string("CUDA error in mg_ce_canon_corr: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}

int mg_ce_canon_destroy(mg_ce_canon* h) {
  free_canon(h);
  return MG_OK;
}

}  // extern "C"

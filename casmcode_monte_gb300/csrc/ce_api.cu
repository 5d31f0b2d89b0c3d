// Host side of the FCC cluster-expansion chain batch: model weights, colouring,
// per-slab site lists, chain parameters, kernel dispatch (C-ABI in montegpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/montegpu.h"
#include "ce_sweep.cuh"
#include "generated/fcc_binary.cuh"
#include "generated/fcc_ternary.cuh"
#include "mg_common.cuh"

namespace mg {

// Adapters from the generated namespaces to the kernel's basis interface.
#define MG_BASIS_ADAPTER(NAME, NS_)                                                       \
  struct NAME {                                                                          \
    static constexpr int NSPECIES = NS_::NSPECIES;                                       \
    static constexpr int NFUNC = NS_::NFUNC;                                             \
    static constexpr int NCLASS = NS_::NCLASS;                                           \
    static constexpr int NFEAT = NS_::NFEAT;                                             \
    static constexpr int HALO = NS_::HALO;                                               \
    __host__ __device__ static constexpr int feat_class(int k) { return NS_::feat_class(k); } \
    __host__ __device__ static constexpr int feat_b(int k) { return NS_::feat_b(k); }     \
    __host__ __device__ static constexpr int psi(int b, int o) { return NS_::psi(b, o); } \
    __host__ __device__ static constexpr int8_t code_of_occ(int o) { return NS_::code_of_occ(o); } \
    __host__ __device__ static constexpr int occ_of_code(int c) { return NS_::occ_of_code(c); } \
    template <class L>                                                                   \
    __device__ static __forceinline__ void features(const L& ld, int (&F)[NFEAT]) {      \
      NS_::features(ld, F);                                                              \
    }                                                                                    \
    template <class L>                                                                   \
    __device__ static __forceinline__ void anchored(const L& ld, long long (&C)[NCLASS]) { \
      NS_::anchored(ld, C);                                                              \
    }                                                                                    \
  };

MG_BASIS_ADAPTER(FccBinary, fcc_binary)
MG_BASIS_ADAPTER(FccTernary, fcc_ternary)
#undef MG_BASIS_ADAPTER

constexpr int NT_BINARY = 512;
constexpr int NT_TERNARY = 256;

// squared pair distances etc. are not needed on the host; multiplicities and the
// decoration scales are derived here from the same generated tables' class counts.
struct ClassInfo {
  long multiplicity;
  double scale;
};

}  // namespace mg

struct mg_ce_model {
  int kind = 0;  // 0 binary, 1 ternary
  int n_species = 2, n_func = 1, n_classes = 0, n_features = 0;
  std::vector<double> eci;
  std::vector<long> mult;
  std::vector<double> scale;
  std::vector<int> feat_class, feat_b;
  std::vector<long> feat_max;  // bound on |F_k|
  std::vector<double> w64;
  std::vector<float> w32;
};

struct mg_ce_batch {
  const mg_ce_model* model = nullptr;
  int L0 = 0, L1 = 0, L2 = 0, n_chains = 0, precision = 0;
  long long N = 0;
  int S = 1, PX = 0, PY = 0, PZ = 0, n_colors = 0, threads = 0;
  size_t smem = 0;
  long long pass = 0;
  std::vector<int32_t> color;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  int8_t* docc = nullptr;
  mg::CeChainParams* dcp = nullptr;
  std::vector<mg::CeChainParams> hcp;
  int* dcstart = nullptr;
  uint32_t* dentries = nullptr;
  uint32_t* dsite = nullptr;
  long long* dout = nullptr;
  size_t out_cap = 0;
};

namespace {

using mg::set_error;

// Class multiplicity and scale (product of site-function scales over the decoration),
// from the generated JSON-equivalent tables compiled below.
#include "generated/fcc_class_tables.inc"

bool make_model(int kind, const double* eci, int n, mg_ce_model* m, std::string& err) {
  m->kind = kind;
  const mg::ClassInfo* info;
  if (kind == 0) {
    m->n_species = mg::FccBinary::NSPECIES;
    m->n_func = mg::FccBinary::NFUNC;
    m->n_classes = mg::FccBinary::NCLASS;
    m->n_features = mg::FccBinary::NFEAT;
    info = kFccBinaryClasses;
    for (int k = 0; k < m->n_features; ++k) {
      m->feat_class.push_back(mg::FccBinary::feat_class(k));
      m->feat_b.push_back(mg::FccBinary::feat_b(k));
      m->feat_max.push_back(kFccBinaryFeatMax[k]);
    }
  } else if (kind == 1) {
    m->n_species = mg::FccTernary::NSPECIES;
    m->n_func = mg::FccTernary::NFUNC;
    m->n_classes = mg::FccTernary::NCLASS;
    m->n_features = mg::FccTernary::NFEAT;
    info = kFccTernaryClasses;
    for (int k = 0; k < m->n_features; ++k) {
      m->feat_class.push_back(mg::FccTernary::feat_class(k));
      m->feat_b.push_back(mg::FccTernary::feat_b(k));
      m->feat_max.push_back(kFccTernaryFeatMax[k]);
    }
  } else {
    err = "Error in mg_ce_model_create: unknown basis_kind";
    return false;
  }
  if (n != m->n_classes) {
    err = "Error in mg_ce_model_create: expected " + std::to_string(m->n_classes) +
          " ECI values, got " + std::to_string(n);
    return false;
  }
  m->eci.assign(eci, eci + n);
  for (int c = 0; c < n; ++c) {
    m->mult.push_back(info[c].multiplicity);
    m->scale.push_back(info[c].scale);
  }
  for (int k = 0; k < m->n_features; ++k) {
    const int f = m->feat_class[k];
    const double w = (m->eci[f] / (double)m->mult[f]) * m->scale[f];
    m->w64.push_back(w);
    m->w32.push_back((float)w);
  }
  return true;
}

int dpsi_max(int kind, int b) {
  if (kind == 0) return 1;
  return b == 0 ? 2 : 3;
}

// Linear colouring colour = (a*i + b*j + c*k) mod m, valid when a*L0, b*L1, c*L2 are
// multiples of m and no neighbour offset maps to 0 mod m; else greedy colouring of the
// periodic conflict graph in lexicographic site order.
std::vector<int32_t> make_coloring(int L0, int L1, int L2, const std::vector<std::array<int, 3>>& offs,
                                   int& n_colors) {
  const long long N = (long long)L0 * L1 * L2;
  std::vector<int32_t> col(N, -1);
  for (int m = 2; m <= 32; ++m) {
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b)
        for (int c = 0; c < m; ++c) {
          if ((1LL * a * L0) % m || (1LL * b * L1) % m || (1LL * c * L2) % m) continue;
          bool ok = true;
          for (auto& o : offs) {
            long long v = (1LL * a * o[0] + 1LL * b * o[1] + 1LL * c * o[2]) % m;
            if (v < 0) v += m;
            if (v == 0) {
              ok = false;
              break;
            }
          }
          if (!ok) continue;
          for (int k = 0; k < L2; ++k)
            for (int j = 0; j < L1; ++j)
              for (int i = 0; i < L0; ++i)
                col[i + (long long)L0 * (j + (long long)L1 * k)] = (int32_t)((1LL * a * i + 1LL * b * j + 1LL * c * k) % m);
          n_colors = m;
          return col;
        }
  }
  // greedy
  n_colors = 0;
  std::vector<char> used;
  for (int k = 0; k < L2; ++k)
    for (int j = 0; j < L1; ++j)
      for (int i = 0; i < L0; ++i) {
        used.assign(64, 0);
        for (auto& o : offs) {
          int a = ((i + o[0]) % L0 + L0) % L0, b = ((j + o[1]) % L1 + L1) % L1, c = ((k + o[2]) % L2 + L2) % L2;
          const int32_t cc = col[a + (long long)L0 * (b + (long long)L1 * c)];
          if (cc >= 0 && cc < 64) used[cc] = 1;
        }
        int cc = 0;
        while (used[cc]) ++cc;
        col[i + (long long)L0 * (j + (long long)L1 * k)] = cc;
        n_colors = std::max(n_colors, cc + 1);
      }
  return col;
}

void free_batch(mg_ce_batch* b) {
  if (!b) return;
  cudaFree(b->docc);
  cudaFree(b->dcp);
  cudaFree(b->dcstart);
  cudaFree(b->dentries);
  cudaFree(b->dsite);
  cudaFree(b->dout);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

template <class B, int NT>
int launch_sweep(mg_ce_batch* bt, int n_passes, long long pass0) {
  mg::CeSweepArgs<B::NFEAT> A;
  A.g.L0 = bt->L0;
  A.g.L1 = bt->L1;
  A.g.L2 = bt->L2;
  A.g.S = bt->S;
  A.g.PX = bt->PX;
  A.g.PY = bt->PY;
  A.g.PZ = bt->PZ;
  A.g.n_colors = bt->n_colors;
  A.g.color_start = bt->dcstart;
  A.g.entries = bt->dentries;
  A.g.site_l = bt->dsite;
  for (int k = 0; k < B::NFEAT; ++k) {
    A.w.w32[k] = bt->model->w32[k];
    A.w.w64[k] = bt->model->w64[k];
  }
  A.cp = bt->dcp;
  A.occ = bt->docc;
  A.pass0 = pass0;
  A.n_passes = n_passes;
  A.n_chains = bt->n_chains;
  A.precision = bt->precision;
  A.out = bt->dout;
  auto kern = mg::ce_sweep_kernel<B, NT>;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt->smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(bt->n_chains * bt->S), 1, 1);
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = bt->smem;
  cfg.stream = bt->stream;
  cudaLaunchAttribute attr[1];
  if (bt->S > 1) {
    if (bt->S > 8) MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)bt->S;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  MG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

template <class B, int NT>
int max_active_clusters(mg_ce_batch* bt, int S, size_t smem, int* out) {
  auto kern = mg::ce_sweep_kernel<B, NT>;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (S > 8) MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  if (S == 1) {
    int nb = 0;
    MG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, NT, smem));
    int dev = 0, sms = 0;
    MG_CUDA_TRY(cudaGetDevice(&dev));
    MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    *out = nb * sms;
    return MG_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(bt->n_chains * S), 1, 1);
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)S;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  MG_CUDA_TRY(cudaOccupancyMaxActiveClusters(&n, (void*)kern, &cfg));
  *out = n;
  return MG_OK;
}

std::vector<std::array<int, 3>> neighbour_offsets(int kind) {
  std::vector<std::array<int, 3>> offs;
  const int* t = kind == 0 ? kFccBinaryOffsets : kFccTernaryOffsets;
  const int n = kind == 0 ? kFccBinaryNOffsets : kFccTernaryNOffsets;
  for (int i = 0; i < n; ++i) offs.push_back({t[3 * i], t[3 * i + 1], t[3 * i + 2]});
  return offs;
}

}  // namespace

extern "C" {

int mg_ce_model_create(int basis_kind, const double* eci, int n_eci, mg_ce_model** out) {
  if (!out || !eci) {
    set_error("Error in mg_ce_model_create: invalid argument");
    return MG_ERR_INVALID;
  }
  auto* m = new mg_ce_model();
  std::string err;
  if (!make_model(basis_kind, eci, n_eci, m, err)) {
    delete m;
    set_error(err);
    return MG_ERR_INVALID;
  }
  *out = m;
  return MG_OK;
}

int mg_ce_model_info(const mg_ce_model* m, int* n_classes, int* n_features, int* n_species) {
  if (!m) {
    set_error("Error in mg_ce_model_info: null model");
    return MG_ERR_INVALID;
  }
  if (n_classes) *n_classes = m->n_classes;
  if (n_features) *n_features = m->n_features;
  if (n_species) *n_species = m->n_species;
  return MG_OK;
}

int mg_ce_model_classes(const mg_ce_model* m, long* multiplicity, double* scale) {
  if (!m) {
    set_error("Error in mg_ce_model_classes: null model");
    return MG_ERR_INVALID;
  }
  for (int c = 0; c < m->n_classes; ++c) {
    if (multiplicity) multiplicity[c] = m->mult[c];
    if (scale) scale[c] = m->scale[c];
  }
  return MG_OK;
}

int mg_ce_model_destroy(mg_ce_model* m) {
  delete m;
  return MG_OK;
}

int mg_ce_batch_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains,
                       const double* temperature, const double* mu, const uint64_t* seeds,
                       const uint32_t* chain_ids, const int8_t* occ, int precision,
                       int ctas_per_chain, mg_ce_batch** out) {
  if (!m || !out || !temperature || !seeds || !occ || n_chains < 1 || (m->n_species > 1 && !mu)) {
    set_error("Error in mg_ce_batch_create: invalid argument");
    return MG_ERR_INVALID;
  }
  if (L0 < 4 || L1 < 4 || L2 < 4) {
    set_error("Error in mg_ce_batch_create: supercell dimensions must be >= 4 (cluster images overlap)");
    return MG_ERR_INVALID;
  }
  if (precision != 0 && precision != 1) {
    set_error("Error in mg_ce_batch_create: precision must be 0 (FP64) or 1 (FP32)");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  if (N > (1LL << 31)) {
    set_error("Error in mg_ce_batch_create: supercell too large");
    return MG_ERR_INVALID;
  }
  for (long long i = 0; i < N * n_chains; ++i)
    if (occ[i] < 0 || occ[i] >= m->n_species) {
      set_error("Error in mg_ce_batch_create: occupant index out of range");
      return MG_ERR_INVALID;
    }
  for (int c = 0; c < n_chains; ++c)
    if (!(temperature[c] > 0.0)) {
      set_error("Error in mg_ce_batch_create: temperature must be > 0");
      return MG_ERR_INVALID;
    }
  auto* b = new mg_ce_batch();
  b->model = m;
  b->L0 = L0;
  b->L1 = L1;
  b->L2 = L2;
  b->N = N;
  b->n_chains = n_chains;
  b->precision = precision;
  const int halo = 2;
  b->PX = L0 + 2 * halo;
  b->PY = L1 + 2 * halo;
  b->threads = m->kind == 0 ? mg::NT_BINARY : mg::NT_TERNARY;

  int dev = 0, sms = 0;
  cudaError_t ce;
  if ((ce = cudaGetDevice(&dev)) != cudaSuccess || (ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
    set_error(std::string("CUDA error in mg_ce_batch_create: ") + cudaGetErrorString(ce));
    delete b;
    return MG_ERR_CUDA;
  }
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t smem_budget = (size_t)max_smem - 1024;  // static accumulators
  // candidate CTAs per chain: every CTA keeps >= halo planes; the largest slab fits
  auto slab_smem = [&](int S) { return (size_t)b->PX * b->PY * ((L2 + S - 1) / S + 2 * halo); };
  std::vector<int> cands;
  for (int S = 1; S <= 16; ++S)
    if (L2 / S >= halo && slab_smem(S) <= smem_budget) cands.push_back(S);
  if (cands.empty()) {
    set_error("Error in mg_ce_batch_create: supercell slab does not fit in shared memory for any CTA count");
    delete b;
    return MG_ERR_INVALID;
  }
  int S = 0;
  if (ctas_per_chain > 0) {
    if (std::find(cands.begin(), cands.end(), ctas_per_chain) == cands.end()) {
      set_error("Error in mg_ce_batch_create: ctas_per_chain must leave >= 2 planes per CTA and fit in shared memory");
      delete b;
      return MG_ERR_INVALID;
    }
    S = ctas_per_chain;
  } else {
    // minimise waves(S) / S, waves = ceil(n_chains / co-resident chains); ties -> fewer CTAs
    double best = 1e300;
    for (int s : cands) {
      int n_active = 0;
      int rc = (m->kind == 0) ? max_active_clusters<mg::FccBinary, mg::NT_BINARY>(b, s, slab_smem(s), &n_active)
                              : max_active_clusters<mg::FccTernary, mg::NT_TERNARY>(b, s, slab_smem(s), &n_active);
      if (rc != MG_OK) {
        delete b;
        return rc;
      }
      if (n_active < 1) continue;
      const double waves = (double)((n_chains + n_active - 1) / n_active);
      const double cost = waves / s;
      if (cost < best * (1.0 - 1e-9)) {
        best = cost;
        S = s;
      }
    }
    if (S == 0) {
      set_error("Error in mg_ce_batch_create: no launchable CTA count for this supercell");
      delete b;
      return MG_ERR_INVALID;
    }
  }
  b->S = S;
  b->PZ = (L2 + S - 1) / S + 2 * halo;
  b->smem = (size_t)b->PX * b->PY * b->PZ;

  // colouring and per-slab, per-colour site lists in bank-interleaved order
  auto offs = neighbour_offsets(m->kind);
  b->color = make_coloring(L0, L1, L2, offs, b->n_colors);
  std::vector<int> cstart((size_t)S * (b->n_colors + 1), 0);
  std::vector<uint32_t> entries, site;
  entries.reserve(N);
  site.reserve(N);
  for (int r = 0; r < S; ++r) {
    const int nk = L2 / S + (r < L2 % S ? 1 : 0);
    const int k0 = r * (L2 / S) + std::min(r, L2 % S);
    for (int c = 0; c < b->n_colors; ++c) {
      cstart[(size_t)r * (b->n_colors + 1) + c] = (int)entries.size();
      std::vector<std::vector<std::pair<uint32_t, uint32_t>>> bank(32);
      for (int kl = 0; kl < nk; ++kl)
        for (int j = 0; j < L1; ++j)
          for (int i = 0; i < L0; ++i) {
            const int k = k0 + kl;
            const long long l = i + (long long)L0 * (j + (long long)L1 * k);
            if (b->color[l] != c) continue;
            const uint32_t pidx = (uint32_t)((i + halo) + b->PX * ((j + halo) + b->PY * (kl + halo)));
            uint32_t flags = 0;
            if (i < halo) flags |= 1;
            else if (i >= L0 - halo) flags |= 2;
            if (j < halo) flags |= 4;
            else if (j >= L1 - halo) flags |= 8;
            if (kl < halo) flags |= 16;
            if (kl >= nk - halo) flags |= 32;
            bank[(pidx >> 2) & 31].push_back({pidx | (flags << 24), (uint32_t)l});
          }
      bool more = true;
      size_t pos = 0;
      while (more) {
        more = false;
        for (int q = 0; q < 32; ++q)
          if (pos < bank[q].size()) {
            entries.push_back(bank[q][pos].first);
            site.push_back(bank[q][pos].second);
            more = true;
          }
        ++pos;
      }
    }
    cstart[(size_t)r * (b->n_colors + 1) + b->n_colors] = (int)entries.size();
  }
  if (b->smem > (size_t)(1u << 24) || entries.size() != (size_t)N) {
    set_error("Error in mg_ce_batch_create: internal site-list construction failed");
    free_batch(b);
    return MG_ERR_INVALID;
  }

  // chain parameters
  const double KB = 8.6173303E-05;
  const int ns = m->n_species;
  b->hcp.resize(n_chains);
  double wsum = 0.0;
  for (int k = 0; k < m->n_features; ++k)
    wsum += std::fabs((double)m->w32[k]) * (double)m->feat_max[k] * dpsi_max(m->kind, m->feat_b[k]);
  for (int c = 0; c < n_chains; ++c) {
    mg::CeChainParams& p = b->hcp[c];
    std::memset(&p, 0, sizeof(p));
    p.beta = 1.0 / (KB * temperature[c]);
    p.beta_log2e = (float)(p.beta * 1.4426950408889634);
    double dmu_max = 0.0;
    for (int o = 0; o < ns; ++o)
      for (int o2 = 0; o2 < ns; ++o2) {
        double r = 0.0;
        for (int i = 0; i < ns - 1; ++i) {
          const double d = (o2 == i + 1 ? 1.0 : 0.0) - (o == i + 1 ? 1.0 : 0.0);
          r += mu[(size_t)c * (ns - 1) + i] * d;
        }
        p.dmu64[o * ns + o2] = r;
        p.dmu32[o * ns + o2] = (float)r;
        dmu_max = std::max(dmu_max, std::fabs(r));
      }
    const double dtol = (m->n_features + 8) * std::ldexp(1.0, -23) * (wsum + dmu_max) + 1e-30;
    p.dtol = (float)(dtol * 1.0001);
    p.eps = (float)(1.25 * p.beta * dtol + 8e-6);
    p.key0 = (uint32_t)seeds[c];
    p.key1 = (uint32_t)(seeds[c] >> 32);
    p.chain_id = chain_ids ? chain_ids[c] : (uint32_t)c;
  }

  auto fail = [&](cudaError_t e, const char* what) {
    set_error(std::string("CUDA error in mg_ce_batch_create: ") + what + ": " + cudaGetErrorString(e));
    free_batch(b);
    return MG_ERR_CUDA;
  };
  cudaError_t e;
#define MGX(expr, what) \
  if ((e = (expr)) != cudaSuccess) return fail(e, what)
  MGX(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
  MGX(cudaEventCreate(&b->ev0), "event");
  MGX(cudaEventCreate(&b->ev1), "event");
  MGX(cudaMalloc(&b->docc, (size_t)N * n_chains), "malloc occ");
  MGX(cudaMalloc(&b->dcp, sizeof(mg::CeChainParams) * n_chains), "malloc params");
  MGX(cudaMalloc(&b->dcstart, sizeof(int) * cstart.size()), "malloc lists");
  MGX(cudaMalloc(&b->dentries, sizeof(uint32_t) * entries.size()), "malloc lists");
  MGX(cudaMalloc(&b->dsite, sizeof(uint32_t) * site.size()), "malloc lists");
  MGX(cudaMemcpyAsync(b->docc, occ, (size_t)N * n_chains, cudaMemcpyHostToDevice, b->stream), "copy");
  MGX(cudaMemcpyAsync(b->dcp, b->hcp.data(), sizeof(mg::CeChainParams) * n_chains, cudaMemcpyHostToDevice, b->stream), "copy");
  MGX(cudaMemcpyAsync(b->dcstart, cstart.data(), sizeof(int) * cstart.size(), cudaMemcpyHostToDevice, b->stream), "copy");
  MGX(cudaMemcpyAsync(b->dentries, entries.data(), sizeof(uint32_t) * entries.size(), cudaMemcpyHostToDevice, b->stream), "copy");
  MGX(cudaMemcpyAsync(b->dsite, site.data(), sizeof(uint32_t) * site.size(), cudaMemcpyHostToDevice, b->stream), "copy");
  MGX(cudaStreamSynchronize(b->stream), "sync");
#undef MGX
  *out = b;
  return MG_OK;
}

int mg_ce_batch_info(const mg_ce_batch* b, int* ctas_per_chain, int* n_colors, int* threads,
                     size_t* smem_bytes) {
  if (!b) {
    set_error("Error in mg_ce_batch_info: null batch");
    return MG_ERR_INVALID;
  }
  if (ctas_per_chain) *ctas_per_chain = b->S;
  if (n_colors) *n_colors = b->n_colors;
  if (threads) *threads = b->threads;
  if (smem_bytes) *smem_bytes = b->smem;
  return MG_OK;
}

int mg_ce_batch_colors(const mg_ce_batch* b, int32_t* color) {
  if (!b || !color) {
    set_error("Error in mg_ce_batch_colors: invalid argument");
    return MG_ERR_INVALID;
  }
  std::memcpy(color, b->color.data(), sizeof(int32_t) * b->color.size());
  return MG_OK;
}

int mg_ce_batch_run(mg_ce_batch* b, int n_passes, long long* out) {
  if (!b || n_passes < 0) {
    set_error("Error in mg_ce_batch_run: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n_passes == 0) return MG_OK;
  const size_t nslot = (size_t)b->model->n_classes + 2;
  const size_t need = (size_t)n_passes * b->n_chains * nslot;
  if (need > b->out_cap) {
    cudaFree(b->dout);
    b->dout = nullptr;
    MG_CUDA_TRY(cudaMalloc(&b->dout, sizeof(long long) * need));
    b->out_cap = need;
  }
  MG_CUDA_TRY(cudaMemsetAsync(b->dout, 0, sizeof(long long) * need, b->stream));
  MG_CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
  int rc = (b->model->kind == 0) ? launch_sweep<mg::FccBinary, mg::NT_BINARY>(b, n_passes, b->pass)
                                 : launch_sweep<mg::FccTernary, mg::NT_TERNARY>(b, n_passes, b->pass);
  if (rc != MG_OK) return rc;
  MG_CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
  if (out) MG_CUDA_TRY(cudaMemcpyAsync(out, b->dout, sizeof(long long) * need, cudaMemcpyDeviceToHost, b->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
  b->pass += n_passes;
  return MG_OK;
}

int mg_ce_batch_last_kernel_ms(const mg_ce_batch* b, float* ms) {
  if (!b || !ms) {
    set_error("Error in mg_ce_batch_last_kernel_ms: invalid argument");
    return MG_ERR_INVALID;
  }
  *ms = b->last_ms;
  return MG_OK;
}

int mg_ce_batch_get_occ(mg_ce_batch* b, int8_t* occ) {
  if (!b || !occ) {
    set_error("Error in mg_ce_batch_get_occ: invalid argument");
    return MG_ERR_INVALID;
  }
  MG_CUDA_TRY(cudaMemcpyAsync(occ, b->docc, (size_t)b->N * b->n_chains, cudaMemcpyDeviceToHost, b->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return MG_OK;
}

int mg_ce_batch_set_occ(mg_ce_batch* b, const int8_t* occ) {
  if (!b || !occ) {
    set_error("Error in mg_ce_batch_set_occ: invalid argument");
    return MG_ERR_INVALID;
  }
  for (long long i = 0; i < b->N * b->n_chains; ++i)
    if (occ[i] < 0 || occ[i] >= b->model->n_species) {
      set_error("Error in mg_ce_batch_set_occ: occupant index out of range");
      return MG_ERR_INVALID;
    }
  MG_CUDA_TRY(cudaMemcpyAsync(b->docc, occ, (size_t)b->N * b->n_chains, cudaMemcpyHostToDevice, b->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return MG_OK;
}

int mg_ce_batch_corr(mg_ce_batch* b, long long* out) {
  if (!b || !out) {
    set_error("Error in mg_ce_batch_corr: invalid argument");
    return MG_ERR_INVALID;
  }
  const int nc = b->model->n_classes;
  long long* d = nullptr;
  MG_CUDA_TRY(cudaMalloc(&d, sizeof(long long) * (size_t)nc * b->n_chains));
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(long long) * (size_t)nc * b->n_chains, b->stream);
  const int nblk = (int)std::min<long long>((b->N + 255) / 256, 1024);
  dim3 grid(nblk, b->n_chains);
  if (e == cudaSuccess) {
    if (b->model->kind == 0)
      mg::ce_corr_kernel<mg::FccBinary><<<grid, 256, 0, b->stream>>>(b->docc, b->L0, b->L1, b->L2, b->n_chains, d);
    else
      mg::ce_corr_kernel<mg::FccTernary><<<grid, 256, 0, b->stream>>>(b->docc, b->L0, b->L1, b->L2, b->n_chains, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, sizeof(long long) * (size_t)nc * b->n_chains, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error(std::string("CUDA error in mg_ce_batch_corr: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}

int mg_ce_batch_delta_e(mg_ce_batch* b, const int32_t* chain, const long long* sites,
                        const int8_t* new_occ, long long n, double* out) {
  if (!b || n < 0 || (n > 0 && (!chain || !sites || !new_occ || !out))) {
    set_error("Error in mg_ce_batch_delta_e: invalid argument");
    return MG_ERR_INVALID;
  }
  if (n == 0) return MG_OK;
  for (long long t = 0; t < n; ++t)
    if (chain[t] < 0 || chain[t] >= b->n_chains || sites[t] < 0 || sites[t] >= b->N || new_occ[t] < 0 ||
        new_occ[t] >= b->model->n_species) {
      set_error("Error in mg_ce_batch_delta_e: proposal out of range");
      return MG_ERR_INVALID;
    }
  int* dc = nullptr;
  long long* ds = nullptr;
  int8_t* dn = nullptr;
  double* dout = nullptr;
  cudaError_t e = cudaMalloc(&dc, sizeof(int) * n);
  if (e == cudaSuccess) e = cudaMalloc(&ds, sizeof(long long) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dn, n);
  if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dc, chain, sizeof(int) * n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ds, sites, sizeof(long long) * n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dn, new_occ, n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) {
    const int nt = 128;
    const unsigned nb = (unsigned)((n + nt - 1) / nt);
    if (b->model->kind == 0) {
      mg::CeWeights<mg::FccBinary::NFEAT> w;
      for (int k = 0; k < mg::FccBinary::NFEAT; ++k) {
        w.w32[k] = b->model->w32[k];
        w.w64[k] = b->model->w64[k];
      }
      mg::ce_delta_e_kernel<mg::FccBinary><<<nb, nt, 0, b->stream>>>(w, b->docc, b->L0, b->L1, b->L2, b->dcp, dc, ds, dn, n, dout);
    } else {
      mg::CeWeights<mg::FccTernary::NFEAT> w;
      for (int k = 0; k < mg::FccTernary::NFEAT; ++k) {
        w.w32[k] = b->model->w32[k];
        w.w64[k] = b->model->w64[k];
      }
      mg::ce_delta_e_kernel<mg::FccTernary><<<nb, nt, 0, b->stream>>>(w, b->docc, b->L0, b->L1, b->L2, b->dcp, dc, ds, dn, n, dout);
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(dc);
  cudaFree(ds);
  cudaFree(dn);
  cudaFree(dout);
  if (e != cudaSuccess) {
    set_error(std::string("CUDA error in mg_ce_batch_delta_e: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}

int mg_ce_batch_destroy(mg_ce_batch* b) {
  free_batch(b);
  return MG_OK;
}

int mg_ce_max_active_chains(const mg_ce_model* m, int L0, int L1, int L2, int ctas_per_chain,
                            int* n_chains) {
  if (!m || !n_chains || L0 < 4 || L1 < 4 || L2 < 4 || ctas_per_chain < 1 || ctas_per_chain > 16 ||
      L2 / ctas_per_chain < 2) {
    set_error("Error in mg_ce_max_active_chains: invalid argument");
    return MG_ERR_INVALID;
  }
  mg_ce_batch tmp;
  tmp.n_chains = 1;
  const size_t smem = (size_t)(L0 + 4) * (L1 + 4) * ((L2 + ctas_per_chain - 1) / ctas_per_chain + 4);
  int rc = (m->kind == 0) ? max_active_clusters<mg::FccBinary, mg::NT_BINARY>(&tmp, ctas_per_chain, smem, n_chains)
                          : max_active_clusters<mg::FccTernary, mg::NT_TERNARY>(&tmp, ctas_per_chain, smem, n_chains);
  return rc;
}

}  // extern "C"

// Host-side helpers of the FCC cluster-expansion sweeps, shared by the chain-batch API
// (ce_api.cu) and the allocation-free entry point (ce_noalloc.cu).  Every helper writes
// into caller-provided buffers and performs no memory allocation of its own.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/montegpu.h"
#include "ce_sweep.cuh"
#include "generated/fcc_binary.cuh"
#include "generated/fcc_ternary.cuh"
#include "mg_common.cuh"

namespace mg {

// Adapters from the generated namespaces to the kernel's basis interface.
#define MG_BASIS_ADAPTER(NAME, NS_, EXTRA)                                                \
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
    EXTRA                                                                                \
  };

// the binary occupation basis also has byte-parallel features (word layout)
#define MG_QUAD_FEATURES                                                                  \
  template <class L>                                                                     \
  __device__ static __forceinline__ void features_quad(const L& ld, uint32_t(&F)[NFEAT]) { \
    fcc_binary::features_quad(ld, F);                                                    \
  }                                                                                      \
  template <int P>                                                                       \
  using Pipe = fcc_binary::Pipe<P>;
// the ternary basis has byte-parallel monomial counts (word layout)
#define MG_TQUAD_COUNTS                                                                   \
  static constexpr int NCOUNT = fcc_ternary::NCOUNT;                                     \
  __host__ __device__ static constexpr int tq_coef(int k, int j) { return fcc_ternary::tq_coef(k, j); } \
  __host__ __device__ static constexpr int tq_const(int k) { return fcc_ternary::tq_const(k); } \
  template <class L>                                                                     \
  __device__ static __forceinline__ void counts_quad(const L& ld, uint32_t(&M)[NCOUNT]) { \
    fcc_ternary::counts_quad(ld, M);                                                     \
  }
MG_BASIS_ADAPTER(FccBinary, fcc_binary, MG_QUAD_FEATURES)
MG_BASIS_ADAPTER(FccTernary, fcc_ternary, MG_TQUAD_COUNTS)
#undef MG_QUAD_FEATURES
#undef MG_TQUAD_COUNTS
#undef MG_BASIS_ADAPTER

constexpr int NT_BINARY = 512;
constexpr int NT_TERNARY = 384;
constexpr int CE_HALO = 2;
constexpr int CE_MAX_COLORS = 64;

struct ClassInfo {
  long multiplicity;
  double scale;
};

namespace host {
#include "generated/fcc_class_tables.inc"
}  // namespace host

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
  // fast-path quantisation: wq[k] = round(w64[k] * 2^qshift); qerr bounds
  // |sum_b dpsi_b sum_k (w64[k] - wq[k] 2^-qshift) F[k]|; qmax bounds |dE_f| of a flip
  std::vector<int32_t> wq;
  int qshift = 0;
  double qerr = 0.0, qmax = 0.0;
  // ternary basis: weights of the monomial counts in the quantised energy sums,
  // sum_k wq[k] F_k = cgc[b] + sum_j cw[b][j] M_j (int32 modulo 2^32), set with wq
  int32_t cw[2][mg::kMaxCounts] = {};
  int32_t cgc[2] = {};
};

namespace mg {
namespace host {

// Codes outside [0, n_species) in occ[0, n), counted into *bad (reads only): the device-side
// admission check of occupations already copied to the device (a host scan of a few MB costs
// more than the copy).
static __global__ void occ_out_of_range_kernel(const int8_t* __restrict__ occ, long long n, int n_species,
                                        unsigned int* __restrict__ bad) {
  unsigned int count = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int o = occ[i];
    count += (o < 0 || o >= n_species) ? 1u : 0u;
  }
  count = __reduce_add_sync(0xffffffffu, count);
  if ((threadIdx.x & 31) == 0 && count) atomicAdd(bad, count);
}

// Process-wide cache of device blocks released by chain batches, per device: a batch of a
// shape seen before takes a released block of at least its size (and at most twice it plus
// 1 MB) instead of cudaMalloc, and its release keeps the block instead of cudaFree (which
// also waits for the whole device).  At most kCacheBlocks blocks and kCacheBytes bytes are
// kept; mg_release_cached_memory frees them.  Callers release a block only after the work
// that used it has finished.
constexpr size_t kCacheBlocks = 8;
constexpr size_t kCacheBytes = size_t(1) << 30;

struct BlockCache {
  std::mutex mu;
  struct Entry {
    int dev;
    void* p;
    size_t bytes;
  };
  std::vector<Entry> blocks;
  size_t total = 0;
};

inline BlockCache& block_cache() {
  static BlockCache* c = new BlockCache();  // never destroyed: batches may outlive static destruction
  return *c;
}

inline cudaError_t cached_malloc(void** p, size_t bytes, size_t* got) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    BlockCache& c = block_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    int best = -1;
    for (int i = 0; i < (int)c.blocks.size(); ++i) {
      const auto& b = c.blocks[i];
      if (b.dev == dev && b.bytes >= bytes && b.bytes <= 2 * bytes + (size_t(1) << 20) &&
          (best < 0 || b.bytes < c.blocks[best].bytes))
        best = i;
    }
    if (best >= 0) {
      *p = c.blocks[best].p;
      *got = c.blocks[best].bytes;
      c.total -= c.blocks[best].bytes;
      c.blocks.erase(c.blocks.begin() + best);
      return cudaSuccess;
    }
  }
  *got = bytes;
  return cudaMalloc(p, bytes);
}

// (dev: the device the block was allocated on, which need not be the current one)
inline void cached_free(void* p, size_t bytes, int dev) {
  if (!p) return;
  {
    BlockCache& c = block_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    if (c.blocks.size() < kCacheBlocks && c.total + bytes <= kCacheBytes) {
      c.blocks.push_back({dev, p, bytes});
      c.total += bytes;
      return;
    }
  }
  cudaFree(p);
}

// Streams of closed batches (a non-blocking stream and two timing events each), kept per
// device like the blocks: creating them costs more than a small job's copies
struct StreamSet {
  int dev;
  cudaStream_t stream;
  cudaEvent_t ev0, ev1;
};

struct StreamCache {
  std::mutex mu;
  std::vector<StreamSet> sets;
};

inline StreamCache& stream_cache() {
  static StreamCache* c = new StreamCache();  // never destroyed, like the block cache
  return *c;
}

inline cudaError_t acquire_stream_set(int dev, StreamSet* out) {
  {
    StreamCache& c = stream_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    for (size_t i = 0; i < c.sets.size(); ++i)
      if (c.sets[i].dev == dev) {
        *out = c.sets[i];
        c.sets.erase(c.sets.begin() + (long)i);
        return cudaSuccess;
      }
  }
  out->dev = dev;
  out->stream = nullptr;
  out->ev0 = out->ev1 = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&out->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&out->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&out->ev1);
  return e;
}

// (the stream has no work left: its batch synchronised it)
inline void release_stream_set(const StreamSet& s) {
  {
    StreamCache& c = stream_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    if (s.stream && s.ev0 && s.ev1 && c.sets.size() < kCacheBlocks) {
      c.sets.push_back(s);
      return;
    }
  }
  if (s.ev0) cudaEventDestroy(s.ev0);
  if (s.ev1) cudaEventDestroy(s.ev1);
  if (s.stream) cudaStreamDestroy(s.stream);
}

inline int release_cached_blocks() {
  {
    StreamCache& sc = stream_cache();
    std::lock_guard<std::mutex> lk(sc.mu);
    for (auto& t : sc.sets) {
      cudaEventDestroy(t.ev0);
      cudaEventDestroy(t.ev1);
      cudaStreamDestroy(t.stream);
    }
    sc.sets.clear();
  }
  BlockCache& c = block_cache();
  std::lock_guard<std::mutex> lk(c.mu);
  cudaError_t first = cudaSuccess;
  for (auto& b : c.blocks) {
    const cudaError_t e = cudaFree(b.p);
    if (first == cudaSuccess) first = e;
  }
  c.blocks.clear();
  c.total = 0;
  if (first != cudaSuccess) {
    set_error(std::string("CUDA error in mg_release_cached_memory: ") + cudaGetErrorString(first));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}

inline int dpsi_max(int kind, int b) {
  if (kind == 0) return 1;
  return b == 0 ? 2 : 3;
}

// Quantised weights of the fast path: the largest shift s (<= 60) for which
// sum_b dpsi_max_b sum_k |w[k]| max|F[k]| 2^s stays below 2^30 (int32 with margin).
inline void quantise_weights(mg_ce_model* m) {
  double T = 0.0;
  for (int k = 0; k < m->n_features; ++k)
    T += dpsi_max(m->kind, m->feat_b[k]) * std::fabs(m->w64[k]) * (double)m->feat_max[k];
  int s = 0;
  while (s < 60 && std::ldexp(T, s + 1) < std::ldexp(1.0, 30)) ++s;
  m->qshift = s;
  m->wq.assign(m->n_features, 0);
  double err = 0.0, qmax = 0.0;
  for (int k = 0; k < m->n_features; ++k) {
    m->wq[k] = (int32_t)std::llround(std::ldexp(m->w64[k], s));
    const double c = dpsi_max(m->kind, m->feat_b[k]) * (double)m->feat_max[k];
    err += c * std::fabs(m->w64[k] - std::ldexp((double)m->wq[k], -s));
    qmax += c * std::fabs(std::ldexp((double)m->wq[k], -s));
  }
  m->qerr = err;
  m->qmax = qmax;
}

template <int NF>
inline void fill_weights(const mg_ce_model* m, CeWeights<NF>& w) {
  for (int k = 0; k < NF; ++k) {
    w.wq[k] = m->wq[k];
    w.w64[k] = m->w64[k];
  }
  w.qscale = (float)std::ldexp(1.0, -m->qshift);
  std::memcpy(w.cw, m->cw, sizeof(w.cw));
  std::memcpy(w.cgc, m->cgc, sizeof(w.cgc));
}

// The count weights of a ternary model (once, when its quantised weights are set: the
// constexpr coefficient tables are cheap in device code, not in a host loop per launch)
inline void set_count_weights(mg_ce_model* m) {
  for (int b = 0; b < 2; ++b) {
    m->cgc[b] = 0;
    for (int j = 0; j < kMaxCounts; ++j) m->cw[b][j] = 0;
  }
  if (m->kind != 1) return;
  long long W[2][FccTernary::NCOUNT] = {}, gc[2] = {};
  for (int k = 0; k < FccTernary::NFEAT; ++k) {
    const int b = FccTernary::feat_b(k);
    gc[b] += (long long)m->wq[k] * FccTernary::tq_const(k);
    for (int j = 0; j < FccTernary::NCOUNT; ++j) W[b][j] += (long long)m->wq[k] * FccTernary::tq_coef(k, j);
  }
  for (int b = 0; b < 2; ++b) {
    m->cgc[b] = (int32_t)(uint32_t)(unsigned long long)gc[b];
    for (int j = 0; j < FccTernary::NCOUNT; ++j) m->cw[b][j] = (int32_t)(uint32_t)(unsigned long long)W[b][j];
  }
}

inline const int* offsets(int kind, int* n) {
  *n = kind == 0 ? kFccBinaryNOffsets : kFccTernaryNOffsets;
  return kind == 0 ? kFccBinaryOffsets : kFccTernaryOffsets;
}

// Colouring of the periodic conflict graph (sites sharing a cluster get different colours).
// Linear colouring (a*i + b*j + c*k) mod m when a*L0, b*L1, c*L2 are multiples of m and no
// neighbour offset maps to 0 mod m (smallest such m); else greedy in lexicographic order.
// Returns the number of colours, or -1 if more than CE_MAX_COLORS would be needed.
// Binary basis: at each m, the colourings of the word-layout pipelines come first (their
// id is returned in *pipe, else -1), then colourings with colour(i + L0/4) = colour(i)
// (the word layout groups the four sites i0 + t*L0/4 of a row).
inline int color_supercell(int L0, int L1, int L2, int kind, int32_t* col, int* pipe = nullptr) {
  int noff = 0;
  const int* off = offsets(kind, &noff);
  const bool want_quad = (kind == 0 || kind == 1) && L0 % 4 == 0;  // both bases have word layouts
  if (pipe) *pipe = -1;
  auto fill_linear = [&](long long a, long long b, long long c, int m) {
    for (int k = 0; k < L2; ++k)
      for (int j = 0; j < L1; ++j)
        for (int i = 0; i < L0; ++i)
          col[i + (long long)L0 * (j + (long long)L1 * k)] = (int32_t)((a * i + b * j + c * k) % m);
  };
  for (int m = 2; m <= 32; ++m) {
    if (want_quad)
      for (int p = 0; p < fcc_binary::NPIPE; ++p) {
        const long long a = fcc_binary::pipe_colouring(p, 0), b = fcc_binary::pipe_colouring(p, 1),
                        c = fcc_binary::pipe_colouring(p, 2);
        if (fcc_binary::pipe_colouring(p, 3) != m) continue;
        if ((a * L0) % m || (b * L1) % m || (c * L2) % m || (a * (L0 / 4)) % m) continue;
        fill_linear(a, b, c, m);
        if (pipe) *pipe = p;
        return m;
      }
    for (int pref = want_quad ? 1 : 0; pref >= 0; --pref)
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b)
        for (int c = 0; c < m; ++c) {
          if ((1LL * a * L0) % m || (1LL * b * L1) % m || (1LL * c * L2) % m) continue;
          if (pref && (1LL * a * (L0 / 4)) % m) continue;
          bool ok = true;
          for (int t = 0; t < noff && ok; ++t) {
            long long v = (1LL * a * off[3 * t] + 1LL * b * off[3 * t + 1] + 1LL * c * off[3 * t + 2]) % m;
            if (v < 0) v += m;
            ok = v != 0;
          }
          if (!ok) continue;
          fill_linear(a, b, c, m);
          return m;
        }
  }
  // greedy: neighbour coordinates from per-axis wrap tables (offsets lie in [-HALO, HALO])
  const long long N = (long long)L0 * L1 * L2;
  for (long long l = 0; l < N; ++l) col[l] = -1;
  const int W = 2 * CE_HALO + 1;
  auto wrap_table = [&](int L, int* t) {
    for (int x = 0; x < L; ++x)
      for (int d = -CE_HALO; d <= CE_HALO; ++d) t[x * W + d + CE_HALO] = ((x + d) % L + L) % L;
  };
  // at most 3 * 128 entries per axis for the sizes accepted here; larger sizes fall back
  // to direct arithmetic
  int ti[1024 * 5], tj[1024 * 5], tk[1024 * 5];
  const bool tables = L0 <= 1024 && L1 <= 1024 && L2 <= 1024;
  if (tables) {
    wrap_table(L0, ti);
    wrap_table(L1, tj);
    wrap_table(L2, tk);
  }
  int n_colors = 0;
  for (int k = 0; k < L2; ++k)
    for (int j = 0; j < L1; ++j)
      for (int i = 0; i < L0; ++i) {
        unsigned long long used = 0ull;  // CE_MAX_COLORS == 64
        for (int t = 0; t < noff; ++t) {
          int a, b, c;
          if (tables) {
            a = ti[i * W + off[3 * t] + CE_HALO];
            b = tj[j * W + off[3 * t + 1] + CE_HALO];
            c = tk[k * W + off[3 * t + 2] + CE_HALO];
          } else {
            a = ((i + off[3 * t]) % L0 + L0) % L0;
            b = ((j + off[3 * t + 1]) % L1 + L1) % L1;
            c = ((k + off[3 * t + 2]) % L2 + L2) % L2;
          }
          const int32_t cc = col[a + (long long)L0 * (b + (long long)L1 * c)];
          if (cc >= 0) used |= 1ull << cc;
        }
        if (used == ~0ull) return -1;
        int cc = 0;
        while (used >> cc & 1ull) ++cc;
        col[i + (long long)L0 * (j + (long long)L1 * k)] = cc;
        n_colors = std::max(n_colors, cc + 1);
      }
  return n_colors;
}

inline int slab_planes(int L2, int S, int r) { return L2 / S + (r < L2 % S ? 1 : 0); }
inline int slab_start(int L2, int S, int r) { return r * (L2 / S) + std::min(r, L2 % S); }
inline size_t slab_smem(int L0, int L1, int L2, int S) {
  return (size_t)(L0 + 2 * CE_HALO) * (L1 + 2 * CE_HALO) * ((L2 + S - 1) / S + 2 * CE_HALO);
}

// Round-robin placement over the 32 shared-memory banks.  Within a bucket of per-bank
// counts cnt[32] the t-th item of bank q goes to offset R_t + #{q2 < q : cnt[q2] > t},
// R_t = sum_q2 min(cnt[q2], t) (all first items of the banks, then all second items, ...):
// a table of these offsets, built once per bucket.
struct BankRoundRobin {
  std::vector<long long> off;  // [t * 32 + q]
  void build(const int* cnt) {
    int tmax = 0;
    for (int q = 0; q < 32; ++q) tmax = std::max(tmax, cnt[q]);
    off.assign((size_t)tmax * 32, 0);
    long long k = 0;
    for (int t = 0; t < tmax; ++t)
      for (int q = 0; q < 32; ++q) {
        off[(size_t)t * 32 + q] = k;
        if (cnt[q] > t) ++k;
      }
  }
  long long at(int q, int t) const { return off[(size_t)t * 32 + q]; }
};

// Per-slab, per-colour site lists (two passes over the slab).  Within one (slab, colour)
// list the sites are grouped
// by (padded index mod 4) and, inside a group, ordered round-robin over the 32 word banks
// ((padded index / 4) mod 32).  Lanes of a warp then share the byte offset within their
// 4-byte word, so every constant neighbour offset keeps their words in distinct banks.
// Entry = padded index | mirror flags << 24 | Philox word << 30; site[e] = Philox counter
// word of the site (see sweep_counter: binary basis with L0 = 4Q: the row's sites
// i0 + tQ share counter i0 + L0 (j + L1 k) and take word t; otherwise counter l, word 0).
// cstart[S][n_colors + 1].
inline void build_site_lists(int L0, int L1, int L2, int S, const int32_t* col, int n_colors, int kind,
                             int* cstart, uint32_t* entries, uint32_t* site) {
  const bool word_rng = kind == 0 && L0 % 4 == 0;
  const int Q = word_rng ? L0 / 4 : L0;
  const int PX = L0 + 2 * CE_HALO, PY = L1 + 2 * CE_HALO;
  // per (colour, residue group, bank): count, then round-robin placement (stack arrays:
  // n_colors <= CE_MAX_COLORS, at most 2^31 sites per bucket)
  int count[CE_MAX_COLORS * 128], seen[CE_MAX_COLORS * 128];
  long long cbase[CE_MAX_COLORS + 1], gbase[CE_MAX_COLORS * 4];
  std::vector<BankRoundRobin> rr((size_t)n_colors * 4);
  long long pos = 0;
  for (int r = 0; r < S; ++r) {
    const int nk = slab_planes(L2, S, r), k0 = slab_start(L2, S, r);
    std::fill(count, count + n_colors * 128, 0);
    std::fill(seen, seen + n_colors * 128, 0);
    for (int kl = 0; kl < nk; ++kl)
      for (int j = 0; j < L1; ++j) {
        const long long row = (long long)L0 * (j + (long long)L1 * (k0 + kl));
        const uint32_t prow = (uint32_t)(CE_HALO + PX * ((j + CE_HALO) + PY * (kl + CE_HALO)));
        for (int i = 0; i < L0; ++i) {
          const uint32_t pidx = prow + i;
          count[(size_t)col[row + i] * 128 + (pidx & 3) * 32 + ((pidx >> 2) & 31)]++;
        }
      }
    cbase[0] = pos;
    for (int c = 0; c < n_colors; ++c) {
      long long b = cbase[c];
      for (int g = 0; g < 4; ++g) {
        gbase[(size_t)c * 4 + g] = b;
        for (int q = 0; q < 32; ++q) b += count[(size_t)c * 128 + g * 32 + q];
      }
      cbase[c + 1] = b;
      cstart[r * (n_colors + 1) + c] = (int)cbase[c];
    }
    cstart[r * (n_colors + 1) + n_colors] = (int)cbase[n_colors];
    for (int b = 0; b < n_colors * 4; ++b) rr[b].build(&count[(size_t)b * 32]);
    for (int kl = 0; kl < nk; ++kl)
      for (int j = 0; j < L1; ++j) {
        const long long row = (long long)L0 * (j + (long long)L1 * (k0 + kl));
        const uint32_t prow = (uint32_t)(CE_HALO + PX * ((j + CE_HALO) + PY * (kl + CE_HALO)));
        for (int i = 0; i < L0; ++i) {
          const long long l = row + i;
          const int c = col[l];
          const uint32_t pidx = prow + i;
          const int g = pidx & 3, q = (pidx >> 2) & 31;
          const int t = seen[(size_t)c * 128 + g * 32 + q]++;
          // round-robin position of the t-th site of bank q within (colour, group)
          const long long p = gbase[(size_t)c * 4 + g] + rr[(size_t)c * 4 + g].at(q, t);
          uint32_t flags = 0;
          if (i < CE_HALO) flags |= 1;
          else if (i >= L0 - CE_HALO) flags |= 2;
          if (j < CE_HALO) flags |= 4;
          else if (j >= L1 - CE_HALO) flags |= 8;
          if (kl < CE_HALO) flags |= 16;
          if (kl >= nk - CE_HALO) flags |= 32;
          const int lane = i / Q;
          entries[p] = pidx | (flags << 24) | ((uint32_t)lane << 30);
          site[p] = (uint32_t)(l - (long long)lane * Q);
        }
      }
    pos = cbase[n_colors];
  }
}

// ---- word layout (four sites per 32-bit word, binary basis)

constexpr int NT_QUAD = 384;
// threads of the ternary word-layout kernel
constexpr int NT_TQUAD = 384;
// threads per role of the warp-specialised kernel: 11 warps, one word per thread (FCC
// 64^3 in 12 row slabs proposes at most 344 words per CTA and colour)
constexpr int NW_WS = 352;

// padded words per row: Q + 2 * HALO, made odd so that consecutive rows start in
// different shared-memory banks
inline int quad_row_stride(int Q) {
  const int r = Q + 2 * CE_HALO;
  return (r & 1) ? r : r + 1;
}
// Row slabs (row_slab) of one kind are valid when every word appears only in its own
// CTA's window (once) and, through the flagged copies, in the previous and the next
// CTA's windows at the offsets dkp and dkn: checked plane by plane over periodic images.
inline bool row_slabs_ok(int L1, int L2, int S, int planes) {
  if (S < 1 || S > L1 * L2 || (planes && S > L2)) return false;
  std::vector<RowSlab> sl(S);
  for (int r = 0; r < S; ++r) {
    sl[r] = row_slab(L1, L2, S, r, planes);
    if (sl[r].r1 <= sl[r].r0) return false;
  }
  for (int r = 0; r < S; ++r) {
    const int prev = (r + S - 1) % S, next = (r + 1) % S;
    const int offp = r == 0 ? L2 : 0, offn = r == S - 1 ? -L2 : 0;
    for (int k = sl[r].kb; k < sl[r].kb + sl[r].nk; ++k)
      for (int x = 0; x < S; ++x)
        for (int off = -2 * L2; off <= 2 * L2; off += L2) {
          const int kk = k + off;
          if (kk < sl[x].kb - CE_HALO || kk > sl[x].kb + sl[x].nk - 1 + CE_HALO) continue;
          const bool expected = (x == r && off == 0) || (x == prev && off == offp) || (x == next && off == offn);
          if (!expected) return false;
        }
  }
  return true;
}
// slab kind of the word layout: balanced rows where valid, else whole planes, else -1
// (memoised: the check walks every periodic image and launches ask for it each time)
inline int word_slab_kind(int L1, int L2, int S) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int>, int> memo;
  const auto key = std::make_tuple(L1, L2, S);
  {
    std::lock_guard<std::mutex> lk(mu);
    const auto it = memo.find(key);
    if (it != memo.end()) return it->second;
  }
  const int kind = row_slabs_ok(L1, L2, S, 0) ? 0 : (row_slabs_ok(L1, L2, S, 1) ? 1 : -1);
  std::lock_guard<std::mutex> lk(mu);
  memo[key] = kind;
  return kind;
}
inline size_t quad_smem(int L0, int L1, int L2, int S) {
  const int kind = word_slab_kind(L1, L2, S);
  return sizeof(uint32_t) * (size_t)quad_row_stride(L0 / 4) * (L1 + 2 * CE_HALO) *
         row_window_planes(L1, L2, S, CE_HALO, kind < 0 ? 1 : kind);
}
// slab decomposition of a layout: row slabs for the word layouts, whole planes (at least
// HALO per CTA) for the byte layout
inline bool slabs_ok(int layout, int L1, int L2, int S) {
  return layout >= 1 ? word_slab_kind(L1, L2, S) >= 0 : (S >= 1 && L2 / S >= CE_HALO);
}
// warp-specialised kernel: the lattice (rounded to 16 bytes) and two stage slots
static_assert(WsStage<FccBinary, 0>::NFIELD == WsStage<FccBinary, 1>::NFIELD, "one stage size for all pipelines");
// warp-specialised kernel: the lattice (rounded to 16 bytes), two stage slots, the CTA's
// site lists (entry and Philox counter word per word) and its colour starts
inline size_t ws_smem(int L0, int L1, int L2, int S, int n_colors = CE_MAX_COLORS) {
  const size_t lattice = (quad_smem(L0, L1, L2, S) + 15) & ~(size_t)15;
  const int kind = word_slab_kind(L1, L2, S);
  const size_t words = (size_t)(L0 / 4) * row_slab_max_rows(L1, L2, S, kind < 0 ? 1 : kind);
  return lattice + sizeof(uint32_t) * (2 * (size_t)WsStage<FccBinary, 0>::NFIELD * NW_WS + 2 * words) +
         sizeof(int) * (n_colors + 1);
}

// The word layout applies when L0 = 4Q with Q >= 4 and the colouring gives the four sites
// i0 + tQ of every row one colour (binary: byte-parallel features; ternary: byte-parallel
// monomial counts).
inline bool quad_eligible(int kind, int L0, int L1, int L2, const int32_t* col) {
  if ((kind != 0 && kind != 1) || L0 % 4 != 0 || L0 / 4 < 4) return false;
  const int Q = L0 / 4;
  const long long rows = (long long)L1 * L2;
  for (long long r = 0; r < rows; ++r) {
    const int32_t* c = col + r * L0;
    for (int i = 0; i < L0 - Q; ++i)
      if (c[i] != c[i + Q]) return false;
  }
  return true;
}

// Per-slab, per-colour word lists of the row slabs (row_slab, kind word_slab_kind; the
// caller has checked that one is valid).  Within one (slab,
// colour) list the words are ordered round-robin over the 32 banks (padded word index mod
// 32), so that the lanes of a warp load from distinct banks at every constant neighbour
// offset.  Entry = padded word index in the slab's window | copy flags << 24 (1: w < 2,
// 2: w >= Q-2, 4: j < 2, 8: j >= L1-2, 16: the word lies in the previous CTA's window,
// 32: in the next CTA's); site[e] = linear index of byte 0's site.
inline void build_word_lists(int L0, int L1, int L2, int S, const int32_t* col, int n_colors, int* cstart,
                             uint32_t* entries, uint32_t* site) {
  const int Q = L0 / 4, RS = quad_row_stride(Q), RY = L1 + 2 * CE_HALO;
  int count[CE_MAX_COLORS * 32], seen[CE_MAX_COLORS * 32];
  long long cbase[CE_MAX_COLORS + 1];
  std::vector<BankRoundRobin> rr(n_colors);
  long long pos = 0;
  const int kind = word_slab_kind(L1, L2, S);
  for (int r = 0; r < S; ++r) {
    const RowSlab sl = row_slab(L1, L2, S, r, kind);
    const RowSlab sp = row_slab(L1, L2, S, (r + S - 1) % S, kind), sn = row_slab(L1, L2, S, (r + 1) % S, kind);
    const int offp = r == 0 ? L2 : 0, offn = r == S - 1 ? -L2 : 0;
    auto prow_of = [&](int j, int k) { return (uint32_t)(CE_HALO + RS * ((j + CE_HALO) + RY * (k - sl.kb + CE_HALO))); };
    std::fill(count, count + n_colors * 32, 0);
    std::fill(seen, seen + n_colors * 32, 0);
    for (int R = sl.r0; R < sl.r1; ++R) {
      const int j = R % L1, k = R / L1;
      const long long row = (long long)L0 * R;
      const uint32_t prow = prow_of(j, k);
      for (int w = 0; w < Q; ++w) count[(size_t)col[row + w] * 32 + ((prow + w) & 31)]++;
    }
    cbase[0] = pos;
    for (int c = 0; c < n_colors; ++c) {
      long long b = cbase[c];
      for (int q = 0; q < 32; ++q) b += count[(size_t)c * 32 + q];
      cbase[c + 1] = b;
      cstart[r * (n_colors + 1) + c] = (int)cbase[c];
    }
    cstart[r * (n_colors + 1) + n_colors] = (int)cbase[n_colors];
    for (int c = 0; c < n_colors; ++c) rr[c].build(&count[(size_t)c * 32]);
    for (int R = sl.r0; R < sl.r1; ++R) {
      const int j = R % L1, k = R / L1;
      const long long row = (long long)L0 * R;
      const uint32_t prow = prow_of(j, k);
      const int kp = k + offp, kn = k + offn;
      const bool in_prev = kp >= sp.kb - CE_HALO && kp <= sp.kb + sp.nk - 1 + CE_HALO;
      const bool in_next = kn >= sn.kb - CE_HALO && kn <= sn.kb + sn.nk - 1 + CE_HALO;
      for (int w = 0; w < Q; ++w) {
        const int c = col[row + w];
        const uint32_t pw = prow + w;
        const int q = pw & 31;
        const int t = seen[(size_t)c * 32 + q]++;
        const long long p = cbase[c] + rr[c].at(q, t);
        uint32_t flags = 0;
        if (w < CE_HALO) flags |= 1;
        else if (w >= Q - CE_HALO) flags |= 2;
        if (j < CE_HALO) flags |= 4;
        else if (j >= L1 - CE_HALO) flags |= 8;
        if (in_prev) flags |= 16;
        if (in_next) flags |= 32;
        entries[p] = pw | (flags << 24);
        site[p] = (uint32_t)(row + w);
      }
    }
    pos = cbase[n_colors];
  }
}

// Chain parameters: beta, Philox key, mu . N dx table and the FP32 error bounds.
inline void make_chain_params(const mg_ce_model* m, int n_chains, const double* temperature,
                              const double* mu, const uint64_t* seeds, const uint32_t* chain_ids,
                              CeChainParams* out) {
  const double KB = 8.6173303E-05;
  const int ns = m->n_species;
  for (int c = 0; c < n_chains; ++c) {
    CeChainParams& p = out[c];
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
    // quantisation error + FP32 rounding of the integer change, of mu.N dx and of the sum
    const double dtol = m->qerr + 2.0 * std::ldexp(1.0, -23) * (m->qmax + dmu_max) + 1e-30;
    p.dtol = (float)(dtol * 1.0001);
    // exp of the quantisation error and of mu.N dx's FP32 rounding, ex2.approx (measured
    // relative error below 2^-22.7 on [-60, 0]; 2^-21 taken), roundings of u and of the band
    // edges (2^-24 + 2^-23); the kernel adds 2e-7 |a| for the roundings that scale with dE32
    p.eps = (float)(1.25 * p.beta * (m->qerr + 1.01 * std::ldexp(dmu_max, -23)) + std::ldexp(1.0, -21) +
                    std::ldexp(1.0, -23) + std::ldexp(1.0, -24) + 1e-8);
    for (int i = 0; i < ns - 1; ++i) p.mu[i] = mu[(size_t)c * (ns - 1) + i];
    p.key0 = (uint32_t)seeds[c];
    p.key1 = (uint32_t)(seeds[c] >> 32);
    p.chain_id = chain_ids ? chain_ids[c] : (uint32_t)c;
  }
}

// Raise a kernel's dynamic shared-memory limit to the most the device allows it (the
// opt-in maximum per CTA less the kernel's static shared memory)
template <class Kern>
int raise_smem_limit(Kern kern) {
  int dev = 0, optin = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  MG_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  return MG_OK;
}

template <class Kern>
int max_active_clusters_query(Kern kern, int NT, int S, size_t smem, int* out) {
  // the limit is raised to the device maximum, never lowered: the occupancy answer depends
  // only on the launch's own shared memory, and a launcher that set the limit once
  // (launch_sweep_ws) keeps a valid limit
  const int rc0 = raise_smem_limit(kern);
  if (rc0 != MG_OK) return rc0;
  if (S > 8) MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  if (S == 1) {
    int nb = 0, dev = 0, sms = 0;
    MG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, NT, smem));
    MG_CUDA_TRY(cudaGetDevice(&dev));
    MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    *out = nb * sms;
    return MG_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)S, 1, 1);
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

template <class Kern>
int max_active_clusters_k(Kern kern, int NT, int S, size_t smem, int* out) {
  // results per (device, kernel, threads, CTAs, shared memory): the query is made once
  static std::mutex mu;
  static std::map<std::tuple<int, const void*, int, int, size_t>, int> cache;
  int dev0 = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev0));
  const auto key = std::make_tuple(dev0, (const void*)kern, NT, S, smem);
  {
    std::lock_guard<std::mutex> lk(mu);
    const auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second;
      return MG_OK;
    }
  }
  const int rc = max_active_clusters_query(kern, NT, S, smem, out);
  if (rc == MG_OK) {
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = *out;
  }
  return rc;
}

// layout 0: one site per byte (ce_sweep_kernel); layout 1: four sites per word
// (ce_sweep_quad_kernel, binary basis); layout 2: the same with pipelined features
inline int max_active_chains(int kind, int S, size_t smem, int* out, int layout = 0) {
  if (layout == 1 && kind == 1)
    return max_active_clusters_k(ce_sweep_tquad_kernel<FccTernary, NT_TQUAD>, NT_TQUAD, S, smem, out);
  if (layout == 1)
    return max_active_clusters_k(ce_sweep_quad_kernel<FccBinary, NT_QUAD, -1>, NT_QUAD, S, smem, out);
  if (layout == 2)
    return max_active_clusters_k(ce_sweep_quad_kernel<FccBinary, NT_QUAD, 0>, NT_QUAD, S, smem, out);
  if (layout == 3)
    return max_active_clusters_k(ce_sweep_ws_kernel<FccBinary, NW_WS, 0>, 2 * NW_WS, S, smem, out);
  return kind == 0 ? max_active_clusters_k(ce_sweep_kernel<FccBinary, NT_BINARY>, NT_BINARY, S, smem, out)
                   : max_active_clusters_k(ce_sweep_kernel<FccTernary, NT_TERNARY>, NT_TERNARY, S, smem, out);
}

inline size_t layout_smem(int layout, int L0, int L1, int L2, int S) {
  if (layout == 3) return ws_smem(L0, L1, L2, S);
  return layout >= 1 ? quad_smem(L0, L1, L2, S) : slab_smem(L0, L1, L2, S);
}

// CTAs per chain: requested (validated) or the S minimising waves(S)/S over the
// launchable candidates (ties -> fewer CTAs).  Returns MG_OK and sets *S_out.
inline int choose_ctas(int kind, int L0, int L1, int L2, int n_chains, int requested, int* S_out, int layout = 0) {
  int dev = 0, max_smem = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t budget = (size_t)max_smem - 1024;
  auto ok = [&](int S) {
    return S >= 1 && S <= 16 && slabs_ok(layout, L1, L2, S) && layout_smem(layout, L0, L1, L2, S) <= budget;
  };
  if (requested > 0) {
    if (!ok(requested)) {
      set_error("Error in ce sweep: ctas_per_chain must leave >= 2 planes per CTA and fit in shared memory");
      return MG_ERR_INVALID;
    }
    *S_out = requested;
    return MG_OK;
  }
  double best = 1e300;
  int S = 0;
  for (int s = 1; s <= 16; ++s) {
    if (!ok(s)) continue;
    int n_active = 0;
    const int rc = max_active_chains(kind, s, layout_smem(layout, L0, L1, L2, s), &n_active, layout);
    if (rc != MG_OK) return rc;
    if (n_active < 1) continue;
    const double cost = (double)((n_chains + n_active - 1) / n_active) / s;
    if (cost < best * (1.0 - 1e-9)) {
      best = cost;
      S = s;
    }
  }
  if (S == 0) {
    set_error("Error in ce sweep: supercell slab does not fit in shared memory for any CTA count");
    return MG_ERR_INVALID;
  }
  *S_out = S;
  return MG_OK;
}

struct SweepLaunch {
  int L0, L1, L2, S, n_colors, n_chains, precision;
  const int* cstart;
  const uint32_t* entries;
  const uint32_t* site;
  const CeChainParams* cp;
  int8_t* occ;
  long long pass0;
  int n_passes;
  long long* out;
  cudaStream_t stream;
  // warp-specialised launches only: launch slot i sweeps chain map_chain[i] from pass
  // pass0 + map_pass[i] (n_map slots, n_map <= CE_MAX_MAP); n_chains stays the batch's
  // chain count (the output stride).  n_map == 0: slot i is chain i, n_chains slots.
  int n_map = 0;
  const int* map_chain = nullptr;
  const int* map_pass = nullptr;
};

template <class B, int NT>
int launch_sweep_t(const mg_ce_model* m, const SweepLaunch& L) {
  CeSweepArgs<B::NFEAT> A;
  A.g.L0 = L.L0;
  A.g.L1 = L.L1;
  A.g.L2 = L.L2;
  A.g.S = L.S;
  A.g.PX = L.L0 + 2 * CE_HALO;
  A.g.PY = L.L1 + 2 * CE_HALO;
  A.g.PZ = (L.L2 + L.S - 1) / L.S + 2 * CE_HALO;
  A.g.n_colors = L.n_colors;
  A.g.color_start = L.cstart;
  A.g.entries = L.entries;
  A.g.site_l = L.site;
  fill_weights(m, A.w);
  A.cp = L.cp;
  A.occ = L.occ;
  A.pass0 = L.pass0;
  A.n_passes = L.n_passes;
  A.n_chains = L.n_chains;
  A.precision = L.precision;
  A.out = L.out;
  const size_t smem = slab_smem(L.L0, L.L1, L.L2, L.S);
  // ternary: four sites per thread and step when a CTA has more than 1.5 sites per thread
  // and colour on average
  auto kern = ce_sweep_kernel<B, NT, kSitesOne>;
  if (B::NSPECIES == 3 && 2 * ((long long)L.L0 * L.L1 * L.L2) > 3LL * NT * L.S * L.n_colors)
    kern = ce_sweep_kernel<B, NT, kSitesFour>;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(L.n_chains * L.S), 1, 1);
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = L.stream;
  cudaLaunchAttribute attr[1];
  if (L.S > 1) {
    if (L.S > 8) MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)L.S;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  MG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

// pipe < 0: generic word-layout kernel; pipe >= 0: pipelined kernel of that colouring
inline int launch_sweep_quad(const mg_ce_model* m, const SweepLaunch& L, int pipe) {
  using B = FccBinary;
  CeQuadArgs<B::NFEAT> A;
  A.g.L0 = L.L0;
  A.g.L1 = L.L1;
  A.g.L2 = L.L2;
  A.g.Q = L.L0 / 4;
  A.g.S = L.S;
  A.g.planes = word_slab_kind(L.L1, L.L2, L.S);
  A.g.window_planes = row_window_planes(L.L1, L.L2, L.S, B::HALO, A.g.planes);
  A.g.max_rows = row_slab_max_rows(L.L1, L.L2, L.S, A.g.planes);
  A.g.RS = quad_row_stride(L.L0 / 4);
  A.g.RY = L.L1 + 2 * CE_HALO;
  A.g.n_colors = L.n_colors;
  A.g.color_start = L.cstart;
  A.g.entries = L.entries;
  A.g.site_l = L.site;
  fill_weights(m, A.w);
  A.cp = L.cp;
  A.occ = L.occ;
  A.pass0 = L.pass0;
  A.n_passes = L.n_passes;
  A.n_chains = L.n_chains;
  A.precision = L.precision;
  A.out = L.out;
  A.n_map = 0;
  const size_t smem = quad_smem(L.L0, L.L1, L.L2, L.S);
  static_assert(fcc_binary::NPIPE == 2, "one kernel instance per pipeline colouring");
  auto kern = pipe == 0 ? ce_sweep_quad_kernel<B, NT_QUAD, 0>
                        : (pipe == 1 ? ce_sweep_quad_kernel<B, NT_QUAD, 1> : ce_sweep_quad_kernel<B, NT_QUAD, -1>);
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(L.n_chains * L.S), 1, 1);
  cfg.blockDim = dim3(NT_QUAD, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = L.stream;
  cudaLaunchAttribute attr[1];
  if (L.S > 1) {
    if (L.S > 8) MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)L.S;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  MG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

// Weights of the ternary word layout from the model's quantised feature weights:
// W[b][j] = sum over features k of basis b of wq[k] tq_coef(k, j), gc[b] = sum wq[k] tq_const(k)
// (modulo 2^32, as the kernel's int32 sums).
inline void fill_tquad_weights(const mg_ce_model* m, TernQuadWeights<FccTernary::NCOUNT>& tw) {
  for (int b = 0; b < 2; ++b) {
    tw.gc[b] = m->cgc[b];
    for (int j = 0; j < FccTernary::NCOUNT; ++j) tw.W[b][j] = m->cw[b][j];
  }
}

// word-layout sweep of the ternary basis
inline int launch_sweep_tquad(const mg_ce_model* m, const SweepLaunch& L) {
  using B = FccTernary;
  CeTQuadArgs<B::NFEAT, B::NCOUNT> TA;
  CeQuadArgs<B::NFEAT>& A = TA.q;
  A.g.L0 = L.L0;
  A.g.L1 = L.L1;
  A.g.L2 = L.L2;
  A.g.Q = L.L0 / 4;
  A.g.S = L.S;
  A.g.planes = word_slab_kind(L.L1, L.L2, L.S);
  A.g.window_planes = row_window_planes(L.L1, L.L2, L.S, B::HALO, A.g.planes);
  A.g.max_rows = row_slab_max_rows(L.L1, L.L2, L.S, A.g.planes);
  A.g.RS = quad_row_stride(L.L0 / 4);
  A.g.RY = L.L1 + 2 * CE_HALO;
  A.g.n_colors = L.n_colors;
  A.g.color_start = L.cstart;
  A.g.entries = L.entries;
  A.g.site_l = L.site;
  fill_weights(m, A.w);
  fill_tquad_weights(m, TA.tw);
  A.cp = L.cp;
  A.occ = L.occ;
  A.pass0 = L.pass0;
  A.n_passes = L.n_passes;
  A.n_chains = L.n_chains;
  A.precision = L.precision;
  A.out = L.out;
  A.n_map = 0;
  const size_t smem = quad_smem(L.L0, L.L1, L.L2, L.S);
  auto kern = ce_sweep_tquad_kernel<B, NT_TQUAD>;
  MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(L.n_chains * L.S), 1, 1);
  cfg.blockDim = dim3(NT_TQUAD, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = L.stream;
  cudaLaunchAttribute attr[1];
  if (L.S > 1) {
    if (L.S > 8) MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)L.S;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  MG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, TA));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

// Words of one chain's window in the grid sweep: the one-slab (S = 1) word window
inline long long tgrid_window_words(int L0, int L1, int L2) {
  return (long long)quad_row_stride(L0 / 4) * (L1 + 2 * CE_HALO) * (L2 + 2 * CE_HALO);
}

// CTAs of the grid sweep that can be resident at once on this device (one cooperative
// launch holds n_chains * G of them)
inline int tgrid_resident_ctas(int* out) {
  int dev = 0, sms = 0, per_sm = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ce_sweep_tgrid_kernel<FccTernary, NT_TQUAD>,
                                                            NT_TQUAD, 0));
  *out = sms * per_sm;
  return MG_OK;
}

// Grid sweep of ternary chains (G CTAs per chain, cooperative launch; lists of the S = 1
// word layout in L.cstart/entries/site; win: n_chains windows of tgrid_window_words words;
// gb: barrier words, zeroed here before the launch)
inline int launch_sweep_tgrid(const mg_ce_model* m, const SweepLaunch& L, int G, uint32_t* win,
                              const GridBarrier& gb, void* gb_block, size_t gb_bytes) {
  using B = FccTernary;
  CeTGridArgs<B::NFEAT, B::NCOUNT> GA;
  CeQuadArgs<B::NFEAT>& A = GA.t.q;
  A.g.L0 = L.L0;
  A.g.L1 = L.L1;
  A.g.L2 = L.L2;
  A.g.Q = L.L0 / 4;
  A.g.S = 1;
  A.g.planes = word_slab_kind(L.L1, L.L2, 1);
  A.g.window_planes = row_window_planes(L.L1, L.L2, 1, B::HALO, A.g.planes);
  A.g.max_rows = row_slab_max_rows(L.L1, L.L2, 1, A.g.planes);
  A.g.RS = quad_row_stride(L.L0 / 4);
  A.g.RY = L.L1 + 2 * CE_HALO;
  A.g.n_colors = L.n_colors;
  A.g.color_start = L.cstart;
  A.g.entries = L.entries;
  A.g.site_l = L.site;
  fill_weights(m, A.w);
  fill_tquad_weights(m, GA.t.tw);
  A.cp = L.cp;
  A.occ = L.occ;
  A.pass0 = L.pass0;
  A.n_passes = L.n_passes;
  A.n_chains = L.n_chains;
  A.precision = L.precision;
  A.out = L.out;
  A.n_map = 0;
  GA.win = win;
  GA.win_words = tgrid_window_words(L.L0, L.L1, L.L2);
  GA.G = G;
  GA.gb = gb;
  MG_CUDA_TRY(cudaMemsetAsync(gb_block, 0, gb_bytes, L.stream));
  void* args[] = {&GA};
  MG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)ce_sweep_tgrid_kernel<B, NT_TQUAD>,
                                          dim3((unsigned)(L.n_chains * G), 1, 1), dim3(NT_TQUAD, 1, 1), args, 0,
                                          L.stream));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

// warp-specialised kernel (pipeline colouring `pipe`, at most NW_WS words per CTA and colour)
inline int launch_sweep_ws(const mg_ce_model* m, const SweepLaunch& L, int pipe) {
  using B = FccBinary;
  CeQuadArgs<B::NFEAT> A;
  A.g.L0 = L.L0;
  A.g.L1 = L.L1;
  A.g.L2 = L.L2;
  A.g.Q = L.L0 / 4;
  A.g.S = L.S;
  A.g.planes = word_slab_kind(L.L1, L.L2, L.S);
  A.g.window_planes = row_window_planes(L.L1, L.L2, L.S, B::HALO, A.g.planes);
  A.g.max_rows = row_slab_max_rows(L.L1, L.L2, L.S, A.g.planes);
  A.g.RS = quad_row_stride(L.L0 / 4);
  A.g.RY = L.L1 + 2 * CE_HALO;
  A.g.n_colors = L.n_colors;
  A.g.color_start = L.cstart;
  A.g.entries = L.entries;
  A.g.site_l = L.site;
  fill_weights(m, A.w);
  A.cp = L.cp;
  A.occ = L.occ;
  A.pass0 = L.pass0;
  A.n_passes = L.n_passes;
  A.n_chains = L.n_chains;
  A.precision = L.precision;
  A.out = L.out;
  if (L.n_map < 0 || L.n_map > CE_MAX_MAP || (L.n_map > 0 && (!L.map_chain || !L.map_pass))) {
    set_error("Error in ce sweep: invalid chain map");
    return MG_ERR_INVALID;
  }
  for (int i = 0; i < L.n_map; ++i)
    if (L.map_chain[i] < 0 || L.map_chain[i] >= L.n_chains || L.map_pass[i] < 0) {
      set_error("Error in ce sweep: invalid chain map");
      return MG_ERR_INVALID;
    }
  A.n_map = L.n_map;
  for (int i = 0; i < CE_MAX_MAP; ++i) {
    A.map_chain[i] = i < L.n_map ? L.map_chain[i] : 0;
    A.map_pass[i] = i < L.n_map ? L.map_pass[i] : 0;
  }
  const int n_slots = L.n_map > 0 ? L.n_map : L.n_chains;
  const size_t smem = ws_smem(L.L0, L.L1, L.L2, L.S, L.n_colors);
  static_assert(fcc_binary::NPIPE == 2, "one kernel instance per pipeline colouring");
  auto kern = pipe == 0 ? ce_sweep_ws_kernel<B, NW_WS, 0> : ce_sweep_ws_kernel<B, NW_WS, 1>;
  {
    // attributes set once per (device, kernel): the device's maximum shared memory (which
    // max_active_clusters_query also sets, never less) and non-portable cluster sizes; a
    // rotated run launches this kernel many times and each call costs host time
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, bool> ready;
    int dev = 0;
    MG_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    bool& done = ready[std::make_pair(dev, (const void*)kern)];
    if (!done) {
      const int rc0 = raise_smem_limit(kern);
      if (rc0 != MG_OK) return rc0;
      MG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      done = true;
    }
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(n_slots * L.S), 1, 1);
  cfg.blockDim = dim3(2 * NW_WS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = L.stream;
  cudaLaunchAttribute attr[1];
  if (L.S > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)L.S;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  MG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A));
  MG_CUDA_TRY(cudaGetLastError());
  return MG_OK;
}

// Integer correlation sums of n_chains chains (out[chain][NCLASS], added to; clear it first):
// the shared-memory tiled recompute (four planes per CTA) where a tile fits, else the
// grid-stride kernel with periodic global loads.
template <class B>
cudaError_t launch_corr(const int8_t* occ, int L0, int L1, int L2, int n_chains, long long* out, cudaStream_t st) {
  constexpr int H = B::HALO;
  static int sm_count[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && sm_count[dev] == 0) {
    e = cudaDeviceGetAttribute(&sm_count[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  const int sms = (dev >= 0 && dev < 64) ? sm_count[dev] : 152;
  // planes per CTA: up to 4, fewer while that leaves under four CTAs per SM (the CTAs are
  // latency-bound: more of them beat the extra halo planes each one loads)
  int nk = std::min(4, L2);
  while (nk > 1 && (long long)((L2 + nk - 1) / nk) * n_chains < 4LL * sms) --nk;
  const size_t smem = (size_t)(L0 + 2 * H) * (L1 + 2 * H) * (nk + 2 * H);
  if (smem <= 200 * 1024) {
    static bool attr_set[64] = {};
    if (smem > 48 * 1024 && dev >= 0 && dev < 64 && !attr_set[dev]) {
      e = cudaFuncSetAttribute(ce_corr_tiled_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      if (e != cudaSuccess) return e;
      attr_set[dev] = true;
    }
    const dim3 grid((unsigned)((L2 + nk - 1) / nk), (unsigned)n_chains);
    ce_corr_tiled_kernel<B><<<grid, 256, smem, st>>>(occ, L0, L1, L2, nk, out);
    return cudaGetLastError();
  }
  const long long N = (long long)L0 * L1 * L2;
  const int nblk = (int)std::min<long long>((N + 255) / 256, 1024);
  ce_corr_kernel<B><<<dim3(nblk, n_chains), 256, 0, st>>>(occ, L0, L1, L2, n_chains, out);
  return cudaGetLastError();
}

inline cudaError_t launch_corr(int kind, const int8_t* occ, int L0, int L1, int L2, int n_chains, long long* out,
                               cudaStream_t st) {
  return kind == 0 ? launch_corr<FccBinary>(occ, L0, L1, L2, n_chains, out, st)
                   : launch_corr<FccTernary>(occ, L0, L1, L2, n_chains, out, st);
}

inline int launch_sweep(const mg_ce_model* m, const SweepLaunch& L) {
  return m->kind == 0 ? launch_sweep_t<FccBinary, NT_BINARY>(m, L) : launch_sweep_t<FccTernary, NT_TERNARY>(m, L);
}

}  // namespace host
}  // namespace mg

// Host side of the FCC cluster-expansion chain batch: model weights, colouring,
// per-slab site lists, chain parameters, kernel dispatch (C-ABI in montegpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/montegpu.h"
#include "ce_host.cuh"
#include "mg_common.cuh"

// Host geometry of one supercell shape, shared by every batch of that shape and built
// once per process: the colouring (number of colours, pipeline colouring id, word-layout
// eligibility) and, per CTA count and layout family (byte / word), the site lists.
struct ShapeColouring {
  std::vector<int32_t> color;
  int n_colors = 0;
  int pipe = -1;
  bool word = false;  // eligible for the word layouts
};
struct ShapeLists {
  std::vector<int> cstart;
  std::vector<uint32_t> entries, site;
  int max_words = 0;  // most words (word lists) or sites of one CTA and colour
};
// Device copies of a shape's site lists on one device, shared by every batch of that shape
// and CTA count (uploaded once per process; freed when evicted from the bounded cache and no
// batch holds them).
struct DeviceLists {
  int* cstart = nullptr;
  uint32_t* entries = nullptr;
  uint32_t* site = nullptr;
  int max_words = 0;
  ~DeviceLists() {
    cudaFree(cstart);
    cudaFree(entries);
    cudaFree(site);
  }
};

struct mg_ce_batch {
  const mg_ce_model* model = nullptr;
  int L0 = 0, L1 = 0, L2 = 0, n_chains = 0, precision = 0;
  long long N = 0;
  int S = 1, PX = 0, PY = 0, PZ = 0, n_colors = 0, threads = 0;
  int layout = 0;  // 0: one site per byte; 1: four sites per word; 2: 1 pipelined; 3: 2 warp-specialised;
                   // 4: word layout swept by the whole grid (ternary)
  int pipe = -1;           // pipeline colouring id of the colouring, or -1
  int ctas_requested = 0;  // 0: chosen by occupancy
  size_t smem = 0;
  long long pass = 0;
  std::shared_ptr<const ShapeColouring> col;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  int last_launches = 0;  // sweep kernels launched by the last run
  // one device allocation holds the occupations, chain parameters, correlation sums of
  // mg_ce_batch_corr and the per-pass outputs of runs of up to kOutPasses passes
  unsigned char* dblock = nullptr;
  size_t dblock_bytes = 0;      // size of the (possibly cached, larger) block
  int dev = 0;                   // device current at creation (owner of the block)
  unsigned int* dbad = nullptr;  // occupant codes out of range found by the creation check
  int8_t* docc = nullptr;
  mg::CeChainParams* dcp = nullptr;
  long long* dcorr = nullptr;
  long long corr_pass = -1;  // pass count at which dcorr holds the current sums (-1: none)
  std::vector<mg::CeChainParams> hcp;
  std::shared_ptr<const DeviceLists> lists;
  int* dcstart = nullptr;
  uint32_t* dentries = nullptr;
  uint32_t* dsite = nullptr;
  long long* dout = nullptr;  // within dblock, or a separate allocation for longer runs
  bool dout_own = false;
  size_t out_cap = 0;
  // Rotation over two cluster sizes (warp-specialised layout with the CTA count chosen by
  // occupancy).  When n_chains - 1 clusters of S_fast > S CTAs fit on the GPU at once but
  // n_chains do not, the chains take turns on one cluster of S CTAs (the slow slot) while
  // the others sweep on clusters of S_fast CTAs, each chain with the call's passes (see
  // rotation_plan).
  int S_fast = 0;  // 0: no rotation
  int rotation_mode = 1;  // 0: never; 1: when the plan beats one unrotated launch; 2: whenever a plan exists
  double launch_passes = 0.0;  // fixed cost of one launch in slow-slot passes (0: not yet measured)
  std::shared_ptr<const DeviceLists> lists_f;
  int* dcstart_f = nullptr;
  uint32_t* dentries_f = nullptr;
  uint32_t* dsite_f = nullptr;
  int max_words = 0, max_words_f = 0;
  double ratio = 1.0;  // time per pass on S_fast CTAs over that on S CTAs (re-measured by rotated calls)
  std::vector<cudaStream_t> stream_fast;  // n_chains - 1 fast lanes, high priority (the batch's
                                          // stream is the slow lane); created by the first
                                          // rotated run
  std::vector<cudaEvent_t> rev;            // six per chain (launch_rotated) and a join
  // grid sweep (layout 4, ternary basis): one allocation holding the barrier words
  // (count[n_chains], gen[n_chains], status, abort) and the chains' windows
  unsigned char* dgrid = nullptr;
  size_t dgrid_bytes = 0, dgrid_bar_bytes = 0;
  mg::GridBarrier gb{};
  uint32_t* dwin = nullptr;
};

// per-pass output rows kept in a batch's own allocation
constexpr int kOutPasses = 128;

// words of one colour per CTA above which a ternary chain is swept by the whole grid
constexpr int kGridWordsPerCta = 1024;

// Pass counts of one rotated call (rotation_plan)
struct RotationPlan {
  std::vector<int> a, g, b;  // chain c: passes on a fast cluster, in the slow slot, fast again
  double makespan = 0.0, unrotated = 0.0;  // simulated, in slow-slot passes
};

namespace {

using mg::set_error;
using namespace mg::host;

// Bounded first-in first-out caches of shape geometry (a shape used again after many
// others is rebuilt).
constexpr size_t kMaxCachedColourings = 32, kMaxCachedLists = 64;
std::mutex g_shape_mu;
std::map<std::tuple<int, int, int, int>, std::shared_ptr<const ShapeColouring>> g_colourings;
std::deque<std::tuple<int, int, int, int>> g_colouring_order;
std::map<std::tuple<int, int, int, int, int, int>, std::shared_ptr<const ShapeLists>> g_lists;
std::deque<std::tuple<int, int, int, int, int, int>> g_lists_order;

// the colouring of a shape; null when it needs more than CE_MAX_COLORS colours
std::shared_ptr<const ShapeColouring> shape_colouring(int kind, int L0, int L1, int L2) {
  const auto key = std::make_tuple(kind, L0, L1, L2);
  {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    const auto it = g_colourings.find(key);
    if (it != g_colourings.end()) return it->second;
  }
  auto c = std::make_shared<ShapeColouring>();
  c->color.assign((size_t)L0 * L1 * L2, -1);
  c->n_colors = color_supercell(L0, L1, L2, kind, c->color.data(), &c->pipe);
  if (c->n_colors < 1) return nullptr;
  c->word = quad_eligible(kind, L0, L1, L2, c->color.data());
  std::lock_guard<std::mutex> lk(g_shape_mu);
  if (g_colourings.emplace(key, c).second) {
    g_colouring_order.push_back(key);
    if (g_colouring_order.size() > kMaxCachedColourings) {
      g_colourings.erase(g_colouring_order.front());
      g_colouring_order.pop_front();
    }
  }
  return g_colourings[key];
}

// site lists of a shape for S CTAs per chain, word (layout >= 1) or byte lists
std::shared_ptr<const ShapeLists> shape_lists(int kind, int L0, int L1, int L2, int S, int layout,
                                              const ShapeColouring& col) {
  const int word = layout >= 1 ? 1 : 0;
  const auto key = std::make_tuple(kind, L0, L1, L2, S, word);
  {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    const auto it = g_lists.find(key);
    if (it != g_lists.end()) return it->second;
  }
  auto l = std::make_shared<ShapeLists>();
  const long long N = (long long)L0 * L1 * L2;
  const long long n_entries = word ? N / 4 : N;
  l->cstart.assign((size_t)S * (col.n_colors + 1), 0);
  l->entries.resize(n_entries);
  l->site.resize(n_entries);
  if (word)
    build_word_lists(L0, L1, L2, S, col.color.data(), col.n_colors, l->cstart.data(), l->entries.data(),
                     l->site.data());
  else
    build_site_lists(L0, L1, L2, S, col.color.data(), col.n_colors, kind, l->cstart.data(), l->entries.data(),
                     l->site.data());
  for (int r = 0; r < S; ++r)
    for (int c = 0; c < col.n_colors; ++c)
      l->max_words = std::max(l->max_words, l->cstart[r * (col.n_colors + 1) + c + 1] - l->cstart[r * (col.n_colors + 1) + c]);
  std::lock_guard<std::mutex> lk(g_shape_mu);
  if (g_lists.emplace(key, l).second) {
    g_lists_order.push_back(key);
    if (g_lists_order.size() > kMaxCachedLists) {
      g_lists.erase(g_lists_order.front());
      g_lists_order.pop_front();
    }
  }
  return g_lists[key];
}

// Device lists per (device, shape, CTA count, list family), uploaded on `st` once per process.
// The cache is never destroyed (no device frees during process exit); at most
// kMaxCachedDeviceLists entries are kept, the oldest dropped first (batches still using an
// entry keep it alive).
constexpr size_t kMaxCachedDeviceLists = 32;
typedef std::tuple<int, int, int, int, int, int, int> DevListKey;
std::map<DevListKey, std::shared_ptr<const DeviceLists>>* g_dev_lists =
    new std::map<DevListKey, std::shared_ptr<const DeviceLists>>();
std::deque<DevListKey>* g_dev_lists_order = new std::deque<DevListKey>();

int device_lists(int kind, int L0, int L1, int L2, int S, int layout, const ShapeColouring& col, cudaStream_t st,
                 std::shared_ptr<const DeviceLists>* out) {
  int dev = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  const DevListKey key = std::make_tuple(dev, kind, L0, L1, L2, S, layout >= 1 ? 1 : 0);
  {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    const auto it = g_dev_lists->find(key);
    if (it != g_dev_lists->end()) {
      *out = it->second;
      return MG_OK;
    }
  }
  const auto host = shape_lists(kind, L0, L1, L2, S, layout, col);
  auto d = std::make_shared<DeviceLists>();
  d->max_words = host->max_words;
  MG_CUDA_TRY(cudaMalloc(&d->cstart, sizeof(int) * host->cstart.size()));
  MG_CUDA_TRY(cudaMalloc(&d->entries, sizeof(uint32_t) * host->entries.size()));
  MG_CUDA_TRY(cudaMalloc(&d->site, sizeof(uint32_t) * host->site.size()));
  MG_CUDA_TRY(cudaMemcpyAsync(d->cstart, host->cstart.data(), sizeof(int) * host->cstart.size(),
                              cudaMemcpyHostToDevice, st));
  MG_CUDA_TRY(cudaMemcpyAsync(d->entries, host->entries.data(), sizeof(uint32_t) * host->entries.size(),
                              cudaMemcpyHostToDevice, st));
  MG_CUDA_TRY(cudaMemcpyAsync(d->site, host->site.data(), sizeof(uint32_t) * host->site.size(),
                              cudaMemcpyHostToDevice, st));
  MG_CUDA_TRY(cudaStreamSynchronize(st));
  std::lock_guard<std::mutex> lk(g_shape_mu);
  auto ins = g_dev_lists->emplace(key, d);
  if (ins.second) {
    g_dev_lists_order->push_back(key);
    if (g_dev_lists_order->size() > kMaxCachedDeviceLists) {
      g_dev_lists->erase(g_dev_lists_order->front());
      g_dev_lists_order->pop_front();
    }
  }
  *out = ins.first->second;
  return MG_OK;
}

bool make_model(int kind, const double* eci, int n, mg_ce_model* m, std::string& err) {
  m->kind = kind;
  const mg::ClassInfo* info;
  if (kind == 0) {
    m->n_species = mg::FccBinary::NSPECIES;
    m->n_func = mg::FccBinary::NFUNC;
    m->n_classes = mg::FccBinary::NCLASS;
    m->n_features = mg::FccBinary::NFEAT;
    info = mg::host::kFccBinaryClasses;
    for (int k = 0; k < m->n_features; ++k) {
      m->feat_class.push_back(mg::FccBinary::feat_class(k));
      m->feat_b.push_back(mg::FccBinary::feat_b(k));
      m->feat_max.push_back(mg::host::kFccBinaryFeatMax[k]);
    }
  } else if (kind == 1) {
    m->n_species = mg::FccTernary::NSPECIES;
    m->n_func = mg::FccTernary::NFUNC;
    m->n_classes = mg::FccTernary::NCLASS;
    m->n_features = mg::FccTernary::NFEAT;
    info = mg::host::kFccTernaryClasses;
    for (int k = 0; k < m->n_features; ++k) {
      m->feat_class.push_back(mg::FccTernary::feat_class(k));
      m->feat_b.push_back(mg::FccTernary::feat_b(k));
      m->feat_max.push_back(mg::host::kFccTernaryFeatMax[k]);
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
  mg::host::quantise_weights(m);
  mg::host::set_count_weights(m);
  return true;
}

// every code of occ[0, n) in [0, n_species): one pass without early exit (vectorisable)
bool occupants_in_range(const int8_t* occ, long long n, int n_species) {
  unsigned bad = 0;
  const unsigned char* u = reinterpret_cast<const unsigned char*>(occ);
  for (long long i = 0; i < n; ++i) bad |= (unsigned)(u[i] >= (unsigned)n_species);
  return bad == 0;
}

void free_batch(mg_ce_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  mg::host::cached_free(b->dblock, b->dblock_bytes, b->dev);
  cudaFree(b->dgrid);
  if (b->dout_own) cudaFree(b->dout);

  for (cudaEvent_t e : b->rev) cudaEventDestroy(e);
  mg::host::release_stream_set(mg::host::StreamSet{b->dev, b->stream, b->ev0, b->ev1});
  for (cudaStream_t s : b->stream_fast) cudaStreamDestroy(s);
  delete b;
}

// Fixed part of a colour phase of the warp-specialised kernel (cluster barrier, loop,
// staging), in words of work per CTA: a phase at S CTAs per chain takes time proportional
// to (most words of one CTA and colour + this).  Fitted on GB300 to 100-pass launches of
// FCC 64^3 at 12 CTAs per chain (342 words, 3.04 ms) and 16 (256 words, 2.62 ms).
constexpr double kWsPhaseFixedWords = 288.0;

// Rotation plan of a warp-specialised batch whose CTA count was chosen by occupancy (the
// fields after out_cap in mg_ce_batch): S_fast is the largest CTA count above S at which
// n_chains - 1 clusters fit at once, kept when the modelled throughput gain,
// ((n_chains - 1) / ratio + 1) / n_chains, is at least 3%.  The slow chain's S-CTA cluster
// runs beside them: on GB300 seven 16-CTA clusters leave a group of 12 SMs that holds one
// 12-CTA cluster (measured: both launches keep their own speed when run together).
int setup_rotation(mg_ce_batch* b) {
  b->lists_f.reset();
  b->dcstart_f = nullptr;
  b->dentries_f = nullptr;
  b->dsite_f = nullptr;
  b->S_fast = 0;
  const int C = b->n_chains;
  if (b->layout != 3 || b->ctas_requested != 0 || b->rotation_mode == 0 || C < 2 || C - 1 > mg::CE_MAX_MAP)
    return MG_OK;
  const mg_ce_model* m = b->model;
  int dev = 0, max_smem = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  MG_CUDA_TRY(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  for (int s = 16; s > b->S; --s) {
    if (!slabs_ok(3, b->L1, b->L2, s)) continue;
    const size_t smem = ws_smem(b->L0, b->L1, b->L2, s);
    if (smem > (size_t)max_smem - 1024) continue;
    int n_active = 0;
    const int rc = max_active_chains(m->kind, s, smem, &n_active, 3);
    if (rc != MG_OK) return rc;
    if (n_active < C - 1) continue;
    const auto lists = shape_lists(m->kind, b->L0, b->L1, b->L2, s, 3, *b->col);
    if (lists->max_words > mg::host::NW_WS) continue;
    const double r = (lists->max_words + kWsPhaseFixedWords) / (b->max_words + kWsPhaseFixedWords);
    if (((C - 1) / r + 1.0) / C < 1.03) break;
    b->S_fast = s;
    b->max_words_f = lists->max_words;
    b->ratio = r;
    break;
  }
  return MG_OK;
}

// Device lists, fast-lane streams and events of a rotated run, made by the batch's first
// rotated run (a batch whose runs are too short to rotate never makes them).
int ensure_rotation_resources(mg_ce_batch* b) {
  const int C = b->n_chains;
  if (!b->lists_f) {
    const int rc = device_lists(b->model->kind, b->L0, b->L1, b->L2, b->S_fast, 3, *b->col, b->stream, &b->lists_f);
    if (rc != MG_OK) return rc;
    b->dcstart_f = b->lists_f->cstart;
    b->dentries_f = b->lists_f->entries;
    b->dsite_f = b->lists_f->site;
  }
  if (b->stream_fast.size() < (size_t)C - 1) {
    int least = 0, greatest = 0;
    MG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    while (b->stream_fast.size() < (size_t)C - 1) {
      cudaStream_t st = nullptr;
      MG_CUDA_TRY(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, greatest));
      b->stream_fast.push_back(st);
    }
  }
  while (b->rev.size() < 6 * (size_t)C + 1) {
    cudaEvent_t e = nullptr;
    MG_CUDA_TRY(cudaEventCreate(&e));
    b->rev.push_back(e);
  }
  return MG_OK;
}

// Fixed cost of one launch of the warp-specialised kernel (prologue, epilogue, launch
// latency) in passes of a chain on the slow cluster, until a rotated call has measured it:
// about 23 us against 31 us per pass of FCC 64^3 at 12 CTAs on GB300.
constexpr double kLaunchFixedPasses = 0.75;

// Pass counts of a rotated call of P passes over C chains and C - 1 fast lanes.  Chain c
// sweeps a_c passes on a fast cluster (lane c; a_0 = 0), then g_c passes in the slow slot
// (chains in order), then b_c passes on a fast cluster again (lane c + 1, after that lane's
// first sweep); the last chain ends in the slow slot (g_{C-1} = P - a_{C-1}).  With r the
// time per pass on a fast cluster over that on the slow one, a_c = round(c g / r) brings
// chain c to the slot as chain c - 1 leaves it; g (every chain but the last) is the value
// whose simulated schedule, with a fixed cost per launch, ends first.  False when no plan
// exists, or (rotation mode 1) when the best plan does not end before one unrotated launch
// of the P passes (P slow passes and one fixed cost): a short call loses more to the extra
// launches than the faster clusters win back.
bool rotation_plan(const mg_ce_batch* b, int P, RotationPlan* plan) {
  const int C = b->n_chains;
  if (b->S_fast <= 0 || P < 2 * C) return false;
  const double r = b->ratio, phi = b->launch_passes > 0.0 ? b->launch_passes : kLaunchFixedPasses;
  double best = 1e300;
  for (int g = 1; g <= P; ++g) {
    std::vector<int> a(C), gg(C), bb(C);
    bool ok = true;
    for (int c = 0; c < C && ok; ++c) {
      a[c] = (int)std::lround(c * (double)g / r);
      gg[c] = c < C - 1 ? g : P - a[c];
      bb[c] = P - a[c] - gg[c];
      ok = a[c] >= 0 && gg[c] >= 1 && bb[c] >= 0;
    }
    if (!ok) continue;
    // simulated schedule in units of a slow-slot pass
    std::vector<double> f1(C, 0.0);
    for (int c = 1; c < C; ++c) f1[c] = a[c] > 0 ? a[c] * r + phi : 0.0;
    double slot = 0.0, end = 0.0;
    for (int c = 0; c < C; ++c) {
      slot = std::max(slot, f1[c]) + gg[c] + phi;
      if (c < C - 1) {
        const double start2 = std::max(slot, f1[c + 1]);
        end = std::max(end, start2 + (bb[c] > 0 ? bb[c] * r + phi : 0.0));
      }
    }
    end = std::max(end, slot);
    if (end < best) {
      best = end;
      plan->a = a;
      plan->g = gg;
      plan->b = bb;
    }
  }
  if (best >= 1e299) return false;
  plan->makespan = best;
  plan->unrotated = P + phi;
  return b->rotation_mode == 2 || best < P + phi;
}

// One chain's sweep of n passes from pass offset `off` of this call, on a cluster of S CTAs
// with the given lists.
int launch_one_chain(mg_ce_batch* b, int chain, int off, int n, int S, const int* cstart, const uint32_t* entries,
                     const uint32_t* site, cudaStream_t st) {
  SweepLaunch L{b->L0, b->L1, b->L2, S, b->n_colors, b->n_chains, b->precision, cstart, entries, site, b->dcp,
                b->docc, b->pass, n, b->dout, st};
  L.n_map = 1;
  L.map_chain = &chain;
  L.map_pass = &off;
  return launch_sweep_ws(b->model, L, b->pipe);
}

// Queue a rotated call (after the output was cleared on b->stream).  Streams: the batch's
// own stream is the slow lane (chains in order); fast lane c (high priority) runs chain c's
// first sweep, then chain c - 1's second sweep.  Every stream receives its commands in the
// planned time order, so that a wait at the head of a hardware queue shared with another
// stream delays only work planned for later; when a fast and a slow sweep become ready
// together the fast cluster, which fits only in a full GPC, is placed first.  Events per
// chain: first fast sweep start/end, slow sweep start/end, second fast sweep start/end.
int launch_rotated(mg_ce_batch* b, const RotationPlan& p) {
  const int C = b->n_chains;
  cudaEvent_t join = b->rev[6 * (size_t)C];
  auto E = [&](int c, int k) { return b->rev[6 * (size_t)c + k]; };
  auto lane = [&](int c) { return b->stream_fast[c - 1]; };
  MG_CUDA_TRY(cudaEventRecord(join, b->stream));
  for (int c = 1; c < C; ++c) {
    MG_CUDA_TRY(cudaStreamWaitEvent(lane(c), join, 0));
    MG_CUDA_TRY(cudaEventRecord(E(c, 0), lane(c)));
    if (p.a[c] > 0) {
      const int rc = launch_one_chain(b, c, 0, p.a[c], b->S_fast, b->dcstart_f, b->dentries_f, b->dsite_f, lane(c));
      if (rc != MG_OK) return rc;
    }
    MG_CUDA_TRY(cudaEventRecord(E(c, 1), lane(c)));
  }
  MG_CUDA_TRY(cudaEventRecord(E(0, 0), b->stream));
  MG_CUDA_TRY(cudaEventRecord(E(0, 1), b->stream));
  for (int c = 0; c < C; ++c) {
    if (c > 0) {
      // chain c - 1's second sweep on lane c, after chain c's first sweep there
      MG_CUDA_TRY(cudaStreamWaitEvent(lane(c), E(c - 1, 3), 0));
      MG_CUDA_TRY(cudaEventRecord(E(c - 1, 4), lane(c)));
      if (p.b[c - 1] > 0) {
        const int rc = launch_one_chain(b, c - 1, p.a[c - 1] + p.g[c - 1], p.b[c - 1], b->S_fast, b->dcstart_f,
                                        b->dentries_f, b->dsite_f, lane(c));
        if (rc != MG_OK) return rc;
      }
      MG_CUDA_TRY(cudaEventRecord(E(c - 1, 5), lane(c)));
      MG_CUDA_TRY(cudaStreamWaitEvent(b->stream, E(c, 1), 0));
    }
    MG_CUDA_TRY(cudaEventRecord(E(c, 2), b->stream));
    const int rc = launch_one_chain(b, c, p.a[c], p.g[c], b->S, b->dcstart, b->dentries, b->dsite, b->stream);
    if (rc != MG_OK) return rc;
    MG_CUDA_TRY(cudaEventRecord(E(c, 3), b->stream));
  }
  MG_CUDA_TRY(cudaEventRecord(E(C - 1, 4), b->stream));
  MG_CUDA_TRY(cudaEventRecord(E(C - 1, 5), b->stream));
  for (int c = 0; c < C - 1; ++c) MG_CUDA_TRY(cudaStreamWaitEvent(b->stream, E(c, 5), 0));
  return MG_OK;
}

// After a rotated call has completed: the time ratio per pass of the two cluster sizes, from
// the first fast sweeps (they start together, before any chain waits for the slow slot)
// and the slow sweeps.  Rotation stops for the batch when it gains nothing (ratio above 1)
// or when the slow cluster evidently did not run beside the fast ones (ratio below 0.6; the
// occupancy model gives 0.86 for FCC 64^3 on GB300).  The fixed cost of a launch comes from
// a least-squares fit of every sweep of the call, t = n t_fast + t0 (fast clusters) or
// n t_slow + t0 (slow slot), expressed in slow-slot passes (t0 / t_slow).
constexpr int kMinRatioPasses = 8;
void update_ratio(mg_ce_batch* b, const RotationPlan& p) {
  const int C = b->n_chains;
  double tf = 0.0, ts = 0.0;
  long nf = 0, ns = 0;
  // normal equations of the fit over unknowns (t_fast, t_slow, t0)
  double A[3][3] = {}, y[3] = {};
  int n_fit = 0;
  auto add = [&](double nfast, double nslow, double t) {
    const double x[3] = {nfast, nslow, 1.0};
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) A[i][j] += x[i] * x[j];
      y[i] += x[i] * t;
    }
    ++n_fit;
  };
  for (int c = 0; c < C; ++c) {
    const cudaEvent_t* e = &b->rev[6 * (size_t)c];
    float ms = 0.f;
    if (c > 0 && p.a[c] > 0 && cudaEventElapsedTime(&ms, e[0], e[1]) == cudaSuccess) {
      add(p.a[c], 0.0, ms);
      // launches of a few passes are dominated by their fixed start-up cost: not in the ratio
      if (p.a[c] >= kMinRatioPasses) {
        tf += ms;
        nf += p.a[c];
      }
    }
    if (cudaEventElapsedTime(&ms, e[2], e[3]) == cudaSuccess) {
      add(0.0, p.g[c], ms);
      if (p.g[c] >= kMinRatioPasses) {
        ts += ms;
        ns += p.g[c];
      }
    }
    if (c < C - 1 && p.b[c] > 0 && cudaEventElapsedTime(&ms, e[4], e[5]) == cudaSuccess) add(p.b[c], 0.0, ms);
  }
  if (nf > 0 && ns > 0 && tf > 0.0 && ts > 0.0) {
    const double r = (tf / nf) / (ts / ns);
    if (r > 1.0 || r < 0.6)
      b->S_fast = 0;
    else
      b->ratio = r;
  }
  if (n_fit >= 4) {
    // Cramer's rule on the 3 x 3 system; kept only when well conditioned and plausible
    auto det3 = [](const double M[3][3]) {
      return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
             M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    };
    const double d = det3(A);
    if (std::fabs(d) > 1e-9) {
      double M[3][3];
      double sol[3];
      for (int k = 0; k < 3; ++k) {
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) M[i][j] = j == k ? y[i] : A[i][j];
        sol[k] = det3(M) / d;
      }
      const double t_slow = sol[1], t0 = sol[2];
      if (t_slow > 0.0 && t0 >= 0.0) b->launch_passes = std::min(std::max(t0 / t_slow, 0.05), 3.0);
    }
  }
}

// Grid sweep (layout 4): the one-slab word lists, G CTAs per chain (requested, else the
// resident CTAs shared evenly between the chains: one cooperative launch holds them all),
// the chains' windows and the barrier words.
int setup_grid(mg_ce_batch* b) {
  const mg_ce_model* m = b->model;
  if (m->kind != 1 || !b->col->word) {
    set_error("Error in mg_ce_batch_set_layout: the grid sweep needs the ternary basis and the word layout");
    return MG_ERR_INVALID;
  }
  int total = 0;
  int rc = mg::host::tgrid_resident_ctas(&total);
  if (rc != MG_OK) return rc;
  const int G = b->ctas_requested > 0 ? b->ctas_requested : total / b->n_chains;
  if (G < 1 || (long long)G * b->n_chains > total) {
    set_error("Error in mg_ce_batch_set_layout: the grid sweep needs all n_chains x ctas_per_chain CTAs resident "
              "at once (" + std::to_string(total) + " on this device)");
    return MG_ERR_INVALID;
  }
  const long long ww = mg::host::tgrid_window_words(b->L0, b->L1, b->L2);
  if (ww >= (1LL << 24)) {
    set_error("Error in mg_ce_batch_set_layout: supercell too large for 24-bit window offsets");
    return MG_ERR_INVALID;
  }
  std::shared_ptr<const DeviceLists> dl;
  rc = device_lists(m->kind, b->L0, b->L1, b->L2, 1, 1, *b->col, b->stream, &dl);
  if (rc != MG_OK) return rc;
  const size_t bar = ((sizeof(unsigned) * 2 * b->n_chains + 2 * sizeof(int)) + 255) & ~(size_t)255;
  const size_t need = bar + sizeof(uint32_t) * (size_t)ww * b->n_chains;
  if (b->dgrid_bytes < need) {
    MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
    cudaFree(b->dgrid);
    b->dgrid = nullptr;
    b->dgrid_bytes = 0;
    MG_CUDA_TRY(cudaMalloc(&b->dgrid, need));
    b->dgrid_bytes = need;
  }
  b->dgrid_bar_bytes = bar;
  b->gb.count = reinterpret_cast<unsigned*>(b->dgrid);
  b->gb.gen = b->gb.count + b->n_chains;
  b->gb.status = reinterpret_cast<int*>(b->gb.gen + b->n_chains);
  b->gb.abort = b->gb.status + 1;
  b->dwin = reinterpret_cast<uint32_t*>(b->dgrid + bar);
  b->lists = dl;
  b->dcstart = dl->cstart;
  b->dentries = dl->entries;
  b->dsite = dl->site;
  b->layout = 4;
  b->S = G;
  b->smem = 0;
  b->PZ = b->L2 + 2 * mg::CE_HALO;
  b->threads = mg::host::NT_TQUAD;
  b->max_words = 0;
  return setup_rotation(b);
}

// CTA count, shared-memory size and site (or word) lists of the batch's layout, uploaded
// to the device (replacing earlier lists).
int setup_layout(mg_ce_batch* b, int layout) {
  const mg_ce_model* m = b->model;
  if (layout == 4) return setup_grid(b);
  int S = 0;
  int rc = choose_ctas(m->kind, b->L0, b->L1, b->L2, b->n_chains, b->ctas_requested, &S, layout);
  if (rc != MG_OK) return rc;
  const size_t smem = layout_smem(layout, b->L0, b->L1, b->L2, S);
  if (smem > (size_t)(1u << 24)) {
    set_error("Error in mg_ce_batch_create: slab too large for 24-bit shared-memory indices");
    return MG_ERR_INVALID;
  }
  const auto lists = shape_lists(m->kind, b->L0, b->L1, b->L2, S, layout, *b->col);
  if (layout == 3 && lists->max_words > mg::host::NW_WS) {
    // the warp-specialised kernel stages at most NW_WS words per (CTA, colour)
    set_error("Error in mg_ce_batch_set_layout: more words per CTA and colour than the warp-specialised "
              "kernel stages");
    return MG_ERR_INVALID;
  }
  std::shared_ptr<const DeviceLists> dl;
  rc = device_lists(m->kind, b->L0, b->L1, b->L2, S, layout, *b->col, b->stream, &dl);
  if (rc != MG_OK) return rc;
  b->lists = dl;
  b->dcstart = dl->cstart;
  b->dentries = dl->entries;
  b->dsite = dl->site;
  b->layout = layout;
  b->S = S;
  b->smem = smem;
  b->PZ = (b->L2 + S - 1) / S + 2 * mg::CE_HALO;
  b->threads = layout == 3 ? 2 * mg::host::NW_WS
                           : (layout >= 1 ? (m->kind == 1 ? mg::host::NT_TQUAD : mg::host::NT_QUAD)
                                          : (m->kind == 0 ? mg::NT_BINARY : mg::NT_TERNARY));
  b->max_words = lists->max_words;
  return setup_rotation(b);
}

}  // namespace

extern "C" {

int mg_release_cached_memory(void) { return mg::host::release_cached_blocks(); }

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
  b->ctas_requested = ctas_per_chain;

  // colouring, then the layout (word layout where the basis and colouring allow it)
  b->col = shape_colouring(m->kind, L0, L1, L2);
  b->n_colors = b->col ? b->col->n_colors : 0;
  b->pipe = b->col ? b->col->pipe : -1;
  if (b->n_colors < 1) {
    set_error("Error in mg_ce_batch_create: colouring needs more than 64 colours");
    delete b;
    return MG_ERR_INVALID;
  }
  // (ternary word layout with more CTAs per chain requested than a cluster holds: the grid sweep)
  const int layout = !b->col->word ? 0
                     : (m->kind == 1 && ctas_per_chain > 16) ? 4
                                                             : ((m->kind == 0 && b->pipe >= 0) ? 3 : 1);
  b->hcp.resize(n_chains);
  make_chain_params(m, n_chains, temperature, mu, seeds, chain_ids, b->hcp.data());

  auto fail = [&](cudaError_t e, const char* what) {
    set_error(std::string("CUDA error in mg_ce_batch_create: ") + what + ": " + cudaGetErrorString(e));
    free_batch(b);
    return MG_ERR_CUDA;
  };
  cudaError_t e;
#define MGX(expr, what) \
  if ((e = (expr)) != cudaSuccess) return fail(e, what)
  MGX(cudaGetDevice(&b->dev), "device");
  {
    mg::host::StreamSet ss;
    e = mg::host::acquire_stream_set(b->dev, &ss);
    b->stream = ss.stream;
    b->ev0 = ss.ev0;
    b->ev1 = ss.ev1;
    MGX(e, "stream");
  }
  {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t nslot = (size_t)m->n_classes + 2;
    const size_t o_cp = al((size_t)N * n_chains);
    const size_t o_corr = o_cp + al(sizeof(mg::CeChainParams) * n_chains);
    const size_t o_bad = o_corr + al(sizeof(long long) * m->n_classes * n_chains);
    const size_t o_out = o_bad + al(sizeof(unsigned int));
    const size_t total = o_out + sizeof(long long) * kOutPasses * n_chains * nslot;
    MGX(mg::host::cached_malloc(reinterpret_cast<void**>(&b->dblock), total, &b->dblock_bytes), "malloc");
    b->dbad = reinterpret_cast<unsigned int*>(b->dblock + o_bad);
    b->docc = reinterpret_cast<int8_t*>(b->dblock);
    b->dcp = reinterpret_cast<mg::CeChainParams*>(b->dblock + o_cp);
    b->dcorr = reinterpret_cast<long long*>(b->dblock + o_corr);
    b->dout = reinterpret_cast<long long*>(b->dblock + o_out);
    b->out_cap = (size_t)kOutPasses * n_chains * nslot;
  }
  MGX(cudaMemcpyAsync(b->docc, occ, (size_t)N * n_chains, cudaMemcpyHostToDevice, b->stream), "copy");
  MGX(cudaMemcpyAsync(b->dcp, b->hcp.data(), sizeof(mg::CeChainParams) * n_chains, cudaMemcpyHostToDevice, b->stream), "copy");
  {
    // occupant codes checked on the device after the copy
    const long long n_occ = N * n_chains;
    const int blocks = (int)std::min<long long>((n_occ + 255) / 256, 1216);
    unsigned int h_bad = 0;
    MGX(cudaMemsetAsync(b->dbad, 0, sizeof(unsigned int), b->stream), "memset");
    mg::host::occ_out_of_range_kernel<<<blocks, 256, 0, b->stream>>>(b->docc, n_occ, m->n_species, b->dbad);
    MGX(cudaGetLastError(), "occupant check");
    MGX(cudaMemcpyAsync(&h_bad, b->dbad, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream), "copy");
    MGX(cudaStreamSynchronize(b->stream), "occupant check");
    if (h_bad != 0) {
      set_error("Error in mg_ce_batch_create: occupant index out of range");
      free_batch(b);
      return MG_ERR_INVALID;
    }
    // the initial correlation sums, which nearly every caller asks for next, computed while
    // the call returns (mg_ce_batch_corr then only copies them back)
    MGX(cudaMemsetAsync(b->dcorr, 0, sizeof(long long) * (size_t)m->n_classes * n_chains, b->stream), "memset");
    MGX(launch_corr(m->kind, b->docc, L0, L1, L2, n_chains, b->dcorr, b->stream), "correlations");
    b->corr_pass = 0;
  }
#undef MGX
  // the best layout that applies; a layout can still be refused for this CTA count (shared
  // memory, staged words), then the next one is tried
  int rc = MG_ERR_INVALID;
  if (layout == 4)
    rc = setup_layout(b, 4);
  else
    for (int lay = layout; lay >= 0 && rc == MG_ERR_INVALID; --lay) {
      if (lay == 1 && layout >= 2) continue;  // a pipeline colouring: layout 2 is always at least as fast
      rc = setup_layout(b, lay);
    }
  // Large ternary chains: when the word window of a 16-CTA cluster does not fit in shared
  // memory (the batch fell back to the byte layout) or a CTA of the cluster layout holds more
  // than kGridWordsPerCta words of one colour, the grid sweep (every resident CTA) is faster
  // (GB300: 128^3 on the byte layout 1261 -> 209 us per pass; 96^3, 864 words per CTA and
  // colour, stays on the cluster: 232 against 253 us) -- provided the grid gives each chain
  // more CTAs than its cluster (152 chains of 48^3 hold one CTA each either way, and their
  // one-CTA word layout is twice as fast as the grid sweep)
  if (rc == MG_OK && m->kind == 1 && b->col->word && ctas_per_chain == 0 &&
      (b->layout == 0 || (b->layout == 1 && b->max_words > kGridWordsPerCta))) {
    int resident = 0;
    if (mg::host::tgrid_resident_ctas(&resident) == MG_OK && resident / n_chains > b->S)
      (void)setup_layout(b, 4);  // refused (too many chains to be resident): stays where it is
  }
  if (rc != MG_OK) {
    free_batch(b);
    return rc;
  }
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

int mg_ce_color_supercell(int basis_kind, int L0, int L1, int L2, int32_t* color, int* word_layout) {
  if (!color || (basis_kind != 0 && basis_kind != 1) || L0 < 4 || L1 < 4 || L2 < 4 ||
      (long long)L0 * L1 * L2 > (1LL << 31)) {
    set_error("Error in mg_ce_color_supercell: invalid argument");
    return -MG_ERR_INVALID;
  }
  int pipe = -1;
  const int n = color_supercell(L0, L1, L2, basis_kind, color, &pipe);
  if (n < 1) {
    set_error("Error in mg_ce_color_supercell: colouring needs more than 64 colours");
    return -MG_ERR_INVALID;
  }
  if (word_layout)
    *word_layout = !quad_eligible(basis_kind, L0, L1, L2, color) ? 0 : ((basis_kind == 0 && pipe >= 0) ? 2 : 1);
  // (a batch may further use layout 3 when its CTA split stages few enough words)
  return n;
}

int mg_ce_batch_layout(const mg_ce_batch* b, int* layout) {
  if (!b || !layout) {
    set_error("Error in mg_ce_batch_layout: invalid argument");
    return MG_ERR_INVALID;
  }
  *layout = b->layout;
  return MG_OK;
}

int mg_ce_batch_set_layout(mg_ce_batch* b, int layout) {
  if (!b || layout < 0 || layout > 4) {
    set_error("Error in mg_ce_batch_set_layout: invalid argument");
    return MG_ERR_INVALID;
  }
  if (layout == 4) return layout == b->layout ? MG_OK : setup_layout(b, 4);
  if (layout >= 1 && !b->col->word) {
    set_error("Error in mg_ce_batch_set_layout: the word layout needs the binary basis, L0 = 4Q with Q >= 4 "
              "and a colouring with colour(i + Q) = colour(i)");
    return MG_ERR_INVALID;
  }
  if (layout >= 2 && b->model->kind != 0) {
    set_error("Error in mg_ce_batch_set_layout: the pipelined and warp-specialised word layouts need the binary "
              "basis");
    return MG_ERR_INVALID;
  }
  if (layout >= 2 && b->pipe < 0) {
    set_error("Error in mg_ce_batch_set_layout: the pipelined word layout needs one of the generated pipeline "
              "colourings");
    return MG_ERR_INVALID;
  }
  if (layout == b->layout) return MG_OK;
  return setup_layout(b, layout);
}

int mg_ce_batch_autotune(mg_ce_batch* b, int probe_passes, int* layout_out, int* ctas_out, float* ms_out) {
  if (!b || probe_passes < 1) {
    set_error("Error in mg_ce_batch_autotune: invalid argument");
    return MG_ERR_INVALID;
  }
  const mg_ce_model* m = b->model;
  const bool word = b->col->word;
  std::vector<int> layouts = {0};
  if (word) layouts.push_back(1);
  if (word && b->pipe >= 0 && m->kind == 0) {
    layouts.push_back(2);
    layouts.push_back(3);
  }
  const int keep_layout = b->layout, keep_req = b->ctas_requested;
  const size_t occ_bytes = (size_t)b->N * b->n_chains;
  int8_t* saved = nullptr;
  MG_CUDA_TRY(cudaMalloc(&saved, occ_bytes));
  cudaError_t e = cudaMemcpyAsync(saved, b->docc, occ_bytes, cudaMemcpyDeviceToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    cudaFree(saved);
    set_error(std::string("CUDA error in mg_ce_batch_autotune: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  float best = 1e30f;
  int best_layout = keep_layout, best_S = b->S;
  const long long pass_keep = b->pass;
  int rc = MG_OK;
  // every layout that applies, each at every CTA count from 1 to 16 that it accepts
  for (int lay : layouts) {
    for (int S = 1; S <= 16 && rc == MG_OK; ++S) {
      b->ctas_requested = S;
      if (setup_layout(b, lay) != MG_OK) continue;  // this CTA count does not fit this layout
      int n_active = 0;
      if (max_active_chains(m->kind, S, b->smem, &n_active, lay) != MG_OK || n_active < 1) continue;
      float ms = 0.f;
      rc = mg_ce_batch_run(b, probe_passes, nullptr);
      if (rc == MG_OK) rc = mg_ce_batch_run(b, probe_passes, nullptr);  // second run timed (warm)
      if (rc != MG_OK) break;
      ms = b->last_ms;
      b->pass = pass_keep;
      e = cudaMemcpyAsync(b->docc, saved, occ_bytes, cudaMemcpyDeviceToDevice, b->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
      if (e != cudaSuccess) {
        rc = MG_ERR_CUDA;
        set_error(std::string("CUDA error in mg_ce_batch_autotune: ") + cudaGetErrorString(e));
        break;
      }
      if (ms < best) {
        best = ms;
        best_layout = lay;
        best_S = S;
      }
    }
  }
  // ternary: the grid sweep with the resident CTAs shared between the chains
  bool best_grid = false;
  if (rc == MG_OK && word && m->kind == 1) {
    b->ctas_requested = 0;
    if (setup_layout(b, 4) == MG_OK) {
      rc = mg_ce_batch_run(b, probe_passes, nullptr);
      if (rc == MG_OK) rc = mg_ce_batch_run(b, probe_passes, nullptr);
      if (rc == MG_OK) {
        const float ms = b->last_ms;
        b->pass = pass_keep;
        e = cudaMemcpyAsync(b->docc, saved, occ_bytes, cudaMemcpyDeviceToDevice, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) {
          rc = MG_ERR_CUDA;
          set_error(std::string("CUDA error in mg_ce_batch_autotune: ") + cudaGetErrorString(e));
        } else if (ms < best) {
          best = ms;
          best_layout = 4;
          best_S = b->S;
          best_grid = true;
        }
      }
    }
  }
  // the occupancy choice of the warp-specialised layout with rotation over two cluster sizes,
  // timed per pass on runs long enough to rotate (at least 4 n_chains passes)
  bool best_rot = false;
  if (rc == MG_OK && word && b->pipe >= 0 && m->kind == 0 && b->rotation_mode != 0) {
    b->ctas_requested = 0;
    if (setup_layout(b, 3) == MG_OK && b->S_fast > 0) {
      const int np = std::max(probe_passes, 4 * b->n_chains);
      rc = mg_ce_batch_run(b, np, nullptr);  // warm; measures the time ratio
      if (rc == MG_OK) rc = mg_ce_batch_run(b, np, nullptr);
      if (rc == MG_OK) {
        const float ms = b->last_ms * (float)probe_passes / (float)np;
        b->pass = pass_keep;
        e = cudaMemcpyAsync(b->docc, saved, occ_bytes, cudaMemcpyDeviceToDevice, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) {
          rc = MG_ERR_CUDA;
          set_error(std::string("CUDA error in mg_ce_batch_autotune: ") + cudaGetErrorString(e));
        } else if (ms < best) {
          best = ms;
          best_layout = 3;
          best_S = b->S;
          best_rot = true;
        }
      }
    }
  }
  cudaFree(saved);
  b->ctas_requested = (best_rot || best_grid) ? 0 : best_S;
  const int rc2 = setup_layout(b, best_layout);
  if (rc != MG_OK) return rc;
  if (rc2 != MG_OK) return rc2;
  (void)keep_req;
  if (layout_out) *layout_out = best_layout;
  if (ctas_out) *ctas_out = best_S;
  if (ms_out) *ms_out = best / (float)probe_passes;
  return MG_OK;
}

int mg_ce_batch_colors(const mg_ce_batch* b, int32_t* color) {
  if (!b || !color) {
    set_error("Error in mg_ce_batch_colors: invalid argument");
    return MG_ERR_INVALID;
  }
  std::memcpy(color, b->col->color.data(), sizeof(int32_t) * b->col->color.size());
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
    if (b->dout_own) cudaFree(b->dout);
    b->dout = nullptr;
    b->dout_own = false;
    MG_CUDA_TRY(cudaMalloc(&b->dout, sizeof(long long) * need));
    b->dout_own = true;
    b->out_cap = need;
  }
  MG_CUDA_TRY(cudaMemsetAsync(b->dout, 0, sizeof(long long) * need, b->stream));
  MG_CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
  SweepLaunch L{b->L0, b->L1, b->L2, b->S, b->n_colors, b->n_chains, b->precision, b->dcstart, b->dentries,
                b->dsite, b->dcp, b->docc, b->pass, n_passes, b->dout, b->stream};
  int rc;
  RotationPlan plan;
  const bool rotated = b->layout == 3 && rotation_plan(b, n_passes, &plan);
  if (rotated) {
    rc = ensure_rotation_resources(b);
    if (rc == MG_OK) rc = launch_rotated(b, plan);
  }
  else if (b->layout == 3)
    rc = launch_sweep_ws(b->model, L, b->pipe);
  else if (b->layout == 4)
    rc = launch_sweep_tgrid(b->model, L, b->S, b->dwin, b->gb, b->dgrid, b->dgrid_bar_bytes);
  else if (b->layout >= 1 && b->model->kind == 1)
    rc = launch_sweep_tquad(b->model, L);
  else if (b->layout >= 1)
    rc = launch_sweep_quad(b->model, L, b->layout == 2 ? b->pipe : -1);
  else
    rc = launch_sweep(b->model, L);
  if (rc != MG_OK) return rc;
  MG_CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
  if (out) MG_CUDA_TRY(cudaMemcpyAsync(out, b->dout, sizeof(long long) * need, cudaMemcpyDeviceToHost, b->stream));
  MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  MG_CUDA_TRY(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
  if (b->layout == 4) {
    int status = 0;
    MG_CUDA_TRY(cudaMemcpy(&status, b->gb.status, sizeof(int), cudaMemcpyDeviceToHost));
    if (status != 0) {
      set_error("Error in mg_ce_batch_run: a grid barrier wait of the sweep ran out; the passes were abandoned "
                "and the occupations left as they were");
      return MG_ERR_DEVICE;
    }
  }
  b->last_launches = 1;
  if (rotated) {
    b->last_launches = b->n_chains;
    for (int c = 0; c < b->n_chains; ++c) b->last_launches += (c > 0 && plan.a[c] > 0) + (plan.b[c] > 0);
    update_ratio(b, plan);
  }
  b->pass += n_passes;
  return MG_OK;
}

int mg_ce_batch_rotation(const mg_ce_batch* b, int* ctas_fast, double* ratio) {
  if (!b) {
    set_error("Error in mg_ce_batch_rotation: invalid argument");
    return MG_ERR_INVALID;
  }
  if (ctas_fast) *ctas_fast = b->S_fast;
  if (ratio) *ratio = b->S_fast > 0 ? b->ratio : 0.0;
  return MG_OK;
}

int mg_ce_batch_rotation_timeline(const mg_ce_batch* b, float* ms) {
  if (!b || !ms) {
    set_error("Error in mg_ce_batch_rotation_timeline: invalid argument");
    return MG_ERR_INVALID;
  }
  if (b->last_launches <= 1 || b->rev.size() < 6 * (size_t)b->n_chains + 1) {
    set_error("Error in mg_ce_batch_rotation_timeline: the last run did not rotate");
    return MG_ERR_INVALID;
  }
  for (int i = 0; i < 6 * b->n_chains; ++i) MG_CUDA_TRY(cudaEventElapsedTime(&ms[i], b->ev0, b->rev[i]));
  return MG_OK;
}

int mg_ce_batch_last_launches(const mg_ce_batch* b, int* launches) {
  if (!b || !launches) {
    set_error("Error in mg_ce_batch_last_launches: invalid argument");
    return MG_ERR_INVALID;
  }
  *launches = b->last_launches;
  return MG_OK;
}

int mg_ce_batch_set_rotation(mg_ce_batch* b, int allowed) {
  if (!b) {
    set_error("Error in mg_ce_batch_set_rotation: invalid argument");
    return MG_ERR_INVALID;
  }
  if (allowed < 0 || allowed > 2) {
    set_error("Error in mg_ce_batch_set_rotation: mode must be 0, 1 or 2");
    return MG_ERR_INVALID;
  }
  b->rotation_mode = allowed;
  return setup_rotation(b);
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
  if (!occupants_in_range(occ, b->N * b->n_chains, b->model->n_species)) {
    set_error("Error in mg_ce_batch_set_occ: occupant index out of range");
    return MG_ERR_INVALID;
  }
  b->corr_pass = -1;
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
  long long* d = b->dcorr;
  cudaError_t e = cudaSuccess;
  if (b->corr_pass != b->pass) {
    e = cudaMemsetAsync(d, 0, sizeof(long long) * (size_t)nc * b->n_chains, b->stream);
    if (e == cudaSuccess) e = launch_corr(b->model->kind, b->docc, b->L0, b->L1, b->L2, b->n_chains, d, b->stream);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, sizeof(long long) * (size_t)nc * b->n_chains, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    set_error(std::string("CUDA error in mg_ce_batch_corr: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  b->corr_pass = b->pass;
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
      mg::host::fill_weights(b->model, w);
      mg::ce_delta_e_kernel<mg::FccBinary><<<nb, nt, 0, b->stream>>>(w, b->docc, b->L0, b->L1, b->L2, b->dcp, dc, ds, dn, n, dout);
    } else {
      mg::CeWeights<mg::FccTernary::NFEAT> w;
      mg::host::fill_weights(b->model, w);
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
  const size_t smem = slab_smem(L0, L1, L2, ctas_per_chain);
  int rc = max_active_chains(m->kind, ctas_per_chain, smem, n_chains);
  return rc;
}

}  // extern "C"

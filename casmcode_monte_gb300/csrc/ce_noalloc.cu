// Allocation-free variant of the coloured cluster-expansion sweep.
//
// Who needs it: callers that cannot call cudaMalloc -- code running inside another
// framework's memory pool or allocator hooks, a process whose device memory is fully
// reserved up front, or a plugin host that forbids allocation during a run.  They own
// the occupation and output buffers; everything else the sweep needs (per-colour site
// lists, per-chain parameters and the occupant-check counter) lives here in a fixed
// file-scope device array, so this entry point calls no cudaMalloc, cudaFree or other
// allocating device routine.  Host staging of the lists and parameters uses static
// arrays; the colouring and site-list helpers still use a little host heap (bank tables,
// the per-device occupancy cache).  Where the CUDA runtime loads modules lazily, the
// first call on a device is when the driver sets up the array's device memory.
//
// The sweep is the byte-layout kernel (one site per byte, any shape), the slowest of the
// library's layouts; the batch API picks faster word layouts where the shape allows.
//
// The caller's occupations are checked on the device before the sweep: a code outside
// [0, n_species) would index outside the kernel's per-species tables.  The check kernel
// counts such codes into the array, the call waits for that count (one synchronisation
// of `stream` per call) and returns an error without sweeping when it is not zero.
//
// Limits: at most MG_NOALLOC_MAX_SITES sites per chain and MG_NOALLOC_MAX_CHAINS chains
// per call; the scratch array (MG_NOALLOC_SCRATCH_BYTES) stays resident on every device
// that loads the library until the process exits.  The first call on a device looks up
// the array's device address with cudaGetSymbolAddress (once per device, with that
// device current), so that first call should come before any stream capture.  All calls
// share the one array and it keeps the last call's contents; calls that overlap on the
// GPU (for example on two streams) race on it, and host calls must not run concurrently.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../include/montegpu.h"
#include "ce_host.cuh"
#include "mg_common.cuh"

namespace {

constexpr long long kMaxSites = MG_NOALLOC_MAX_SITES;
constexpr int kMaxChains = MG_NOALLOC_MAX_CHAINS;
constexpr int kMaxCtas = 16;
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffCp = 0;
constexpr size_t kOffCstart = align256(kOffCp + sizeof(mg::CeChainParams) * kMaxChains);
constexpr size_t kOffEntries = align256(kOffCstart + sizeof(int) * kMaxCtas * (mg::CE_MAX_COLORS + 1));
constexpr size_t kOffSite = align256(kOffEntries + sizeof(uint32_t) * kMaxSites);
constexpr size_t kOffBad = align256(kOffSite + sizeof(uint32_t) * kMaxSites);
constexpr size_t kScratchBytes = align256(kOffBad + sizeof(unsigned int));
static_assert(kScratchBytes <= MG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

// The scratch array.  Host code must not use its name as an address (it is a host-side
// stand-in); the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_sweep_scratch[MG_NOALLOC_SCRATCH_BYTES];

// per-device address of g_sweep_scratch (set on the first call on that device)
static unsigned char* g_scratch_dev[kMaxDevices] = {};

// host staging, static so that no host heap is used either
static mg::CeChainParams h_cp[kMaxChains];
static int h_cstart[kMaxCtas * (mg::CE_MAX_COLORS + 1)];
static uint32_t h_entries[kMaxSites];
static uint32_t h_site[kMaxSites];
static int32_t h_color[kMaxSites];
static unsigned int h_bad = 0;

// Counts occupant codes outside [0, n_species) in occ[0, n) into *bad.  Reads only.
__global__ void occupant_check_kernel(const int8_t* __restrict__ occ, long long n, int n_species,
                                      unsigned int* __restrict__ bad) {
  unsigned int count = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int o = occ[i];
    count += (o < 0 || o >= n_species) ? 1u : 0u;
  }
  count = __reduce_add_sync(0xffffffffu, count);
  if ((threadIdx.x & 31) == 0 && count) atomicAdd(bad, count);
}

int scratch_address(unsigned char** out) {
  int dev = 0;
  MG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    mg::set_error("Error in mg_ce_sweep_noalloc: device index beyond 64");
    return MG_ERR_INVALID;
  }
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    MG_CUDA_TRY(cudaGetSymbolAddress(&p, g_sweep_scratch));
    g_scratch_dev[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_dev[dev];
  return MG_OK;
}

}  // namespace

extern "C" int mg_ce_sweep_noalloc(const mg_ce_model* m, int L0, int L1, int L2, int n_chains,
                                   const double* temperature, const double* mu,
                                   const uint64_t* seeds, int8_t* d_occ, long long pass0,
                                   int n_passes, long long* d_out, int precision, void* stream) {
  using namespace mg::host;
  if (!m || !temperature || !seeds || !d_occ || !d_out || (m->n_species > 1 && !mu) || n_passes < 1 ||
      pass0 < 0 || n_chains < 1 || (precision != 0 && precision != 1)) {
    mg::set_error("Error in mg_ce_sweep_noalloc: invalid argument");
    return MG_ERR_INVALID;
  }
  if (L0 < 4 || L1 < 4 || L2 < 4) {
    mg::set_error("Error in mg_ce_sweep_noalloc: supercell dimensions must be >= 4");
    return MG_ERR_INVALID;
  }
  const long long N = (long long)L0 * L1 * L2;
  if (N > kMaxSites) {
    mg::set_error("Error in mg_ce_sweep_noalloc: supercell has more than MG_NOALLOC_MAX_SITES (262144) sites");
    return MG_ERR_INVALID;
  }
  if (n_chains > kMaxChains) {
    mg::set_error("Error in mg_ce_sweep_noalloc: more than MG_NOALLOC_MAX_CHAINS (64) chains");
    return MG_ERR_INVALID;
  }
  for (int c = 0; c < n_chains; ++c)
    if (!(temperature[c] > 0.0)) {
      mg::set_error("Error in mg_ce_sweep_noalloc: temperature must be > 0");
      return MG_ERR_INVALID;
    }
  unsigned char* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != MG_OK) return rc;
  int S = 0;
  rc = choose_ctas(m->kind, L0, L1, L2, n_chains, 0, &S);
  if (rc != MG_OK) return rc;
  const int n_colors = color_supercell(L0, L1, L2, m->kind, h_color);
  if (n_colors < 1) {
    mg::set_error("Error in mg_ce_sweep_noalloc: colouring needs more than 64 colours");
    return MG_ERR_INVALID;
  }
  build_site_lists(L0, L1, L2, S, h_color, n_colors, m->kind, h_cstart, h_entries, h_site);
  make_chain_params(m, n_chains, temperature, mu, seeds, nullptr, h_cp);

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // occupant codes first: nothing is swept unless every code is in range
  unsigned int* d_bad = reinterpret_cast<unsigned int*>(scratch + kOffBad);
  MG_CUDA_TRY(cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), st));
  const long long n_occ = N * n_chains;
  const int check_blocks = (int)std::min<long long>((n_occ + 255) / 256, 1184);
  occupant_check_kernel<<<check_blocks, 256, 0, st>>>(d_occ, n_occ, m->n_species, d_bad);
  MG_CUDA_TRY(cudaGetLastError());
  MG_CUDA_TRY(cudaMemcpyAsync(&h_bad, d_bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
  MG_CUDA_TRY(cudaStreamSynchronize(st));
  if (h_bad != 0) {
    mg::set_error("Error in mg_ce_sweep_noalloc: occupant index out of range (" + std::to_string(h_bad) +
                  " codes outside [0, n_species))");
    return MG_ERR_INVALID;
  }
  mg::CeChainParams* d_cp = reinterpret_cast<mg::CeChainParams*>(scratch + kOffCp);
  int* d_cstart = reinterpret_cast<int*>(scratch + kOffCstart);
  uint32_t* d_entries = reinterpret_cast<uint32_t*>(scratch + kOffEntries);
  uint32_t* d_site = reinterpret_cast<uint32_t*>(scratch + kOffSite);
  // pageable sources are staged by the driver before these calls return, so the static
  // host arrays may be rewritten by the next call
  MG_CUDA_TRY(cudaMemcpyAsync(d_cp, h_cp, sizeof(mg::CeChainParams) * n_chains, cudaMemcpyHostToDevice, st));
  MG_CUDA_TRY(cudaMemcpyAsync(d_cstart, h_cstart, sizeof(int) * S * (n_colors + 1), cudaMemcpyHostToDevice, st));
  MG_CUDA_TRY(cudaMemcpyAsync(d_entries, h_entries, sizeof(uint32_t) * N, cudaMemcpyHostToDevice, st));
  MG_CUDA_TRY(cudaMemcpyAsync(d_site, h_site, sizeof(uint32_t) * N, cudaMemcpyHostToDevice, st));
  // per-pass outputs are accumulated with atomics: clear the caller's buffer first
  const size_t out_bytes = sizeof(long long) * (size_t)n_passes * n_chains * (m->n_classes + 2);
  MG_CUDA_TRY(cudaMemsetAsync(d_out, 0, out_bytes, st));
  SweepLaunch L{L0, L1, L2, S, n_colors, n_chains, precision, d_cstart, d_entries, d_site,
                d_cp, d_occ, pass0, n_passes, d_out, st};
  return launch_sweep(m, L);
}

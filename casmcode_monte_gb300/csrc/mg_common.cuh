// Shared device helpers: Philox4x32-10, mt19937_64 (warp-parallel regeneration),
// error plumbing for the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace mg {

// ---- error handling (host) ----
void set_error(const std::string& msg);
const char* last_error();

#define MG_CUDA_TRY(expr)                                                                 \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess) {                                                              \
      ::mg::set_error(std::string("CUDA error in ") + __func__ + ": " + #expr + ": " +   \
                      cudaGetErrorString(_e));                                            \
      return 2;                                                                           \
    }                                                                                     \
  } while (0)

// ---- Philox4x32-10 (Salmon et al., SC'11; the Random123 definition) ----
struct U32x4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ U32x4 philox4x32_10(U32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
#ifdef __CUDA_ARCH__
    const uint32_t lo0 = 0xD2511F53u * c.x;
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
#else
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    c = U32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

//: stream tag of the semi-grand canonical sweep (4th counter word)
constexpr uint32_t SWEEP_TAG = 0x4D434753u;

// ---- mt19937_64 (Matsumoto & Nishimura; parameters of [rand.predef] mt19937_64) ----
constexpr int MT_N = 312;
constexpr int MT_M = 156;
constexpr uint64_t MT_A = 0xB5026F5AA96619E9ull;
constexpr uint64_t MT_UPPER = 0xFFFFFFFF80000000ull;
constexpr uint64_t MT_LOWER = 0x000000007FFFFFFFull;

__host__ __device__ __forceinline__ uint64_t mt_temper(uint64_t z) {
  z ^= (z >> 29) & 0x5555555555555555ull;
  z ^= (z << 17) & 0x71D67FFFEDA60000ull;
  z ^= (z << 37) & 0xFFF7EEE000000000ull;
  z ^= (z >> 43);
  return z;
}

// One warp regenerates the 312-word state in place.  Element i depends on x[i], x[i+1]
// and x[i+156] (all mod 312) with the sequential order of the reference generator; the
// two halves [0,156) and [156,312) are each done in chunks of 32 with read-before-write.
__device__ __forceinline__ void mt_twist_warp(uint64_t* x, int lane) {
#pragma unroll 1
  for (int half = 0; half < 2; ++half) {
    const int base = half * MT_M;
#pragma unroll 1
    for (int c0 = 0; c0 < MT_M; c0 += 32) {
      const int i = base + c0 + lane;
      const bool act = (c0 + lane) < MT_M;
      uint64_t v = 0;
      if (act) {
        const uint64_t y = (x[i] & MT_UPPER) | (x[(i + 1) % MT_N] & MT_LOWER);
        v = x[(i + MT_M) % MT_N] ^ (y >> 1) ^ ((y & 1ull) ? MT_A : 0ull);
      }
      __syncwarp();
      if (act) x[i] = v;
      __syncwarp();
    }
  }
}

// Lemire's nearly-divisionless bounded integer in [0, range) from 64-bit words
// ("Fast Random Integer Generation in an Interval", ACM TOMACS 29(1), 2019), the method
// libstdc++ uses for std::uniform_int_distribution over a 64-bit engine.
struct Lemire64 {
  uint64_t range;      // b - a + 1
  uint64_t threshold;  // (2^64 - range) mod range
};

}  // namespace mg

// Shared device helpers: Philox4x32-10, mt19937_64 (warp-parallel regeneration),
// error plumbing for the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <sstream>
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

// Text form of a mt19937_64 state as libstdc++'s operator<< / operator>> write and read it:
// the 312 state words, then the position index, separated by spaces.
inline int parse_mt_state(const char* text, uint64_t* out313) {
  std::istringstream ss(text);
  for (int i = 0; i < MT_N + 1; ++i) {
    unsigned long long v;
    if (!(ss >> v)) return -1;
    out313[i] = v;
  }
  return 0;
}

inline std::string format_mt_state(const uint64_t* s313) {
  std::ostringstream ss;
  for (int i = 0; i < MT_N; ++i) ss << (unsigned long long)s313[i] << ' ';
  ss << (unsigned long long)s313[MT_N];
  return ss.str();
}

// next tempered word of a warp-shared state (x: 312 words in shared memory, p: position,
// uniform across the warp); the warp regenerates the state when it is used up
__device__ __forceinline__ uint64_t mt_next_warp(uint64_t* x, int& p, int lane) {
  if (p >= MT_N) {
    mt_twist_warp(x, lane);
    p = 0;
  }
  const uint64_t y = x[p];
  p += 1;
  return mt_temper(y);
}

// std::uniform_int_distribution<64-bit>(0, range - 1) over mt19937_64 as libstdc++
// computes it for a range below 2^64: Lemire's method with a 128-bit product, drawing again
// while the low half is below (2^64 - range) mod range.
__device__ __forceinline__ uint64_t mt_uniform_int_warp(uint64_t* x, int& p, int lane, uint64_t range) {
  uint64_t w = mt_next_warp(x, p, lane);
  uint64_t lo = w * range;
  uint64_t hi = __umul64hi(w, range);
  if (lo < range) {
    const uint64_t threshold = (0ull - range) % range;
    while (lo < threshold) {
      w = mt_next_warp(x, p, lane);
      lo = w * range;
      hi = __umul64hi(w, range);
    }
  }
  return hi;
}

// std::generate_canonical<double, 53>(mt19937_64) as libstdc++ computes it: one word,
// double(word) / 2^64 (exact scaling of the rounded word), and the largest double below 1
// if that rounds up to 1.
__device__ __forceinline__ double mt_canonical_warp(uint64_t* x, int& p, int lane) {
  const uint64_t w = mt_next_warp(x, p, lane);
  double u = __dmul_rn(__ull2double_rn(w), 5.421010862427522170e-20);
  if (u >= 1.0) u = 0.99999999999999988898;
  return u;
}

// Lemire's nearly-divisionless bounded integer in [0, range) from 64-bit words
// ("Fast Random Integer Generation in an Interval", ACM TOMACS 29(1), 2019), the method
// libstdc++ uses for std::uniform_int_distribution over a 64-bit engine.
struct Lemire64 {
  uint64_t range;      // b - a + 1
  uint64_t threshold;  // (2^64 - range) mod range
};

}  // namespace mg

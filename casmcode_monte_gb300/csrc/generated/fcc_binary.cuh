// Generated by casmcode_monte_gb300/clex/codegen.py -- do not edit.
// Basis set 'fcc_binary': 10 classes, 9 local features,
// 54 neighbour offsets (FCC 1-4NN pairs, 3 smallest triplets, NN tetrahedron).
#pragma once
#include <cstdint>
namespace mg { namespace fcc_binary {
constexpr int NSPECIES = 2;
constexpr int NFUNC = 1;
constexpr int NCLASS = 10;
constexpr int NFEAT = 9;
constexpr int NOFF = 54;
constexpr int HALO = 2;
__host__ __device__ constexpr int feat_class(int k) {
  constexpr int t[NFEAT] = {1, 2, 3, 4, 5, 6, 7, 8, 9};
  return t[k];
}
__host__ __device__ constexpr int feat_b(int k) {
  constexpr int t[NFEAT] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  return t[k];
}
__host__ __device__ constexpr int psi0(int o) {
  constexpr int t[NSPECIES] = {0, 1};
  return t[o];
}
__host__ __device__ __forceinline__ constexpr int psi(int b, int o) { return o; }
__host__ __device__ constexpr int8_t code_of_occ(int o) { return (int8_t)o; }
__host__ __device__ constexpr int occ_of_code(int c) { return c; }
// F[k] = sum over decorated clusters (class feat_class(k), basis feat_b(k) at the
// changing site) of the product of the other sites' integer psi values.
template <class Loader>
__device__ __forceinline__ void features(const Loader& ld, int (&F)[NFEAT]) {
  const int v_m2_0_0 = ld(-2, 0, 0);
  const int v_m2_0_1 = ld(-2, 0, 1);
  const int v_m2_0_2 = ld(-2, 0, 2);
  const int v_m2_1_0 = ld(-2, 1, 0);
  const int v_m2_1_1 = ld(-2, 1, 1);
  const int v_m2_2_0 = ld(-2, 2, 0);
  const int v_m1_m1_0 = ld(-1, -1, 0);
  const int v_m1_m1_1 = ld(-1, -1, 1);
  const int v_m1_m1_2 = ld(-1, -1, 2);
  const int v_m1_0_m1 = ld(-1, 0, -1);
  const int v_m1_0_0 = ld(-1, 0, 0);
  const int v_m1_0_1 = ld(-1, 0, 1);
  const int v_m1_0_2 = ld(-1, 0, 2);
  const int v_m1_1_m1 = ld(-1, 1, -1);
  const int v_m1_1_0 = ld(-1, 1, 0);
  const int v_m1_1_1 = ld(-1, 1, 1);
  const int v_m1_2_m1 = ld(-1, 2, -1);
  const int v_m1_2_0 = ld(-1, 2, 0);
  const int v_0_m2_0 = ld(0, -2, 0);
  const int v_0_m2_1 = ld(0, -2, 1);
  const int v_0_m2_2 = ld(0, -2, 2);
  const int v_0_m1_m1 = ld(0, -1, -1);
  const int v_0_m1_0 = ld(0, -1, 0);
  const int v_0_m1_1 = ld(0, -1, 1);
  const int v_0_m1_2 = ld(0, -1, 2);
  const int v_0_0_m2 = ld(0, 0, -2);
  const int v_0_0_m1 = ld(0, 0, -1);
  const int v_0_0_1 = ld(0, 0, 1);
  const int v_0_0_2 = ld(0, 0, 2);
  const int v_0_1_m2 = ld(0, 1, -2);
  const int v_0_1_m1 = ld(0, 1, -1);
  const int v_0_1_0 = ld(0, 1, 0);
  const int v_0_1_1 = ld(0, 1, 1);
  const int v_0_2_m2 = ld(0, 2, -2);
  const int v_0_2_m1 = ld(0, 2, -1);
  const int v_0_2_0 = ld(0, 2, 0);
  const int v_1_m2_0 = ld(1, -2, 0);
  const int v_1_m2_1 = ld(1, -2, 1);
  const int v_1_m1_m1 = ld(1, -1, -1);
  const int v_1_m1_0 = ld(1, -1, 0);
  const int v_1_m1_1 = ld(1, -1, 1);
  const int v_1_0_m2 = ld(1, 0, -2);
  const int v_1_0_m1 = ld(1, 0, -1);
  const int v_1_0_0 = ld(1, 0, 0);
  const int v_1_0_1 = ld(1, 0, 1);
  const int v_1_1_m2 = ld(1, 1, -2);
  const int v_1_1_m1 = ld(1, 1, -1);
  const int v_1_1_0 = ld(1, 1, 0);
  const int v_2_m2_0 = ld(2, -2, 0);
  const int v_2_m1_m1 = ld(2, -1, -1);
  const int v_2_m1_0 = ld(2, -1, 0);
  const int v_2_0_m2 = ld(2, 0, -2);
  const int v_2_0_m1 = ld(2, 0, -1);
  const int v_2_0_0 = ld(2, 0, 0);
  F[0] = 1;
  F[1] = ((v_m1_0_0 + v_0_m1_1 + v_0_1_0) + (v_m1_0_1 + v_0_0_m1 + v_1_m1_0)) + ((v_m1_1_0 + v_0_0_1 + v_1_0_m1) + (v_0_m1_0 + v_0_1_m1 + v_1_0_0));
  F[2] = ((v_m1_m1_1 + v_1_m1_1) + (v_m1_1_m1 + v_1_1_m1)) + ((v_m1_1_1) + (v_1_m1_m1));
  F[3] = ((v_m2_0_1 + v_m1_m1_2 + v_m1_2_0 + v_0_1_m2 + v_1_m2_1 + v_1_1_0) + (v_m2_1_0 + v_m1_0_m1 + v_0_m2_1 + v_0_1_1 + v_1_0_m2 + v_2_m1_m1)) + ((v_m2_1_1 + v_m1_0_2 + v_0_m1_m1 + v_0_2_m1 + v_1_0_1 + v_2_m1_0) + (v_m1_m1_0 + v_m1_2_m1 + v_0_m1_2 + v_1_m2_0 + v_1_1_m2 + v_2_0_m1));
  F[4] = ((v_m2_0_0 + v_0_m2_2 + v_0_2_0) + (v_m2_0_2 + v_0_0_m2 + v_2_m2_0)) + ((v_m2_2_0 + v_0_0_2 + v_2_0_m2) + (v_0_m2_0 + v_0_2_m2 + v_2_0_0));
  F[5] = ((v_m1_0_0 * v_m1_0_1 + v_m1_0_1 * v_m1_1_0 + v_m1_1_0 * v_0_1_0 + v_0_m1_1 * v_0_0_1 + v_0_0_1 * v_0_1_0 + v_0_1_0 * v_1_0_0) + (v_m1_0_0 * v_m1_1_0 + v_m1_0_1 * v_0_m1_1 + v_0_m1_0 * v_0_m1_1 + v_0_m1_1 * v_1_m1_0 + v_0_0_1 * v_1_0_0 + v_1_m1_0 * v_1_0_m1)) + ((v_m1_0_0 * v_0_m1_0 + v_m1_0_1 * v_0_0_1 + v_0_m1_0 * v_0_0_m1 + v_0_0_m1 * v_0_1_m1 + v_0_1_m1 * v_0_1_0 + v_1_m1_0 * v_1_0_0) + (v_m1_0_0 * v_0_0_m1 + v_m1_1_0 * v_0_1_m1 + v_0_m1_0 * v_1_m1_0 + v_0_0_m1 * v_1_0_m1 + v_0_1_m1 * v_1_0_m1 + v_1_0_m1 * v_1_0_0));
  F[6] = ((v_m1_m1_1 * v_m1_0_0 + v_m1_0_0 * v_m1_1_m1 + v_m1_0_1 * v_0_m1_0 + v_m1_1_m1 * v_0_1_m1 + v_m1_1_1 * v_0_0_1 + v_0_m1_1 * v_1_m1_1 + v_0_0_1 * v_1_m1_0 + v_0_1_0 * v_1_0_m1 + v_1_m1_0 * v_1_m1_1) + (v_m1_m1_1 * v_m1_0_1 + v_m1_0_0 * v_0_m1_1 + v_m1_0_1 * v_0_1_0 + v_m1_1_0 * v_m1_1_1 + v_m1_1_1 * v_0_1_0 + v_0_m1_1 * v_1_0_0 + v_0_0_1 * v_1_m1_1 + v_0_1_0 * v_1_1_m1 + v_1_m1_1 * v_1_0_0)) + ((v_m1_m1_1 * v_0_m1_0 + v_m1_0_0 * v_0_1_m1 + v_m1_1_m1 * v_m1_1_0 + v_m1_1_0 * v_0_0_m1 + v_0_m1_0 * v_1_m1_m1 + v_0_0_m1 * v_1_m1_m1 + v_0_1_m1 * v_1_0_0 + v_1_m1_m1 * v_1_m1_0 + v_1_0_m1 * v_1_1_m1) + (v_m1_m1_1 * v_0_m1_1 + v_m1_0_1 * v_m1_1_1 + v_m1_1_m1 * v_0_0_m1 + v_m1_1_0 * v_0_0_1 + v_0_m1_0 * v_1_0_m1 + v_0_0_m1 * v_1_m1_0 + v_0_1_m1 * v_1_1_m1 + v_1_m1_m1 * v_1_0_m1 + v_1_0_0 * v_1_1_m1));
  F[7] = ((v_m2_0_1 * v_m1_0_0 + v_m2_1_1 * v_m1_0_1 + v_m1_m1_2 * v_m1_0_1 + v_m1_0_0 * v_0_0_1 + v_m1_0_1 * v_m1_0_2 + v_m1_0_1 * v_1_0_0 + v_m1_1_0 * v_0_m1_0 + v_m1_2_m1 * v_0_1_m1 + v_0_m1_m1 * v_0_m1_0 + v_0_m1_0 * v_1_m2_0 + v_0_m1_1 * v_0_1_0 + v_0_0_m1 * v_0_1_m2 + v_0_0_1 * v_0_1_m1 + v_0_1_m2 * v_0_1_m1 + v_0_1_0 * v_0_1_1 + v_1_m2_0 * v_1_m1_0 + v_1_0_m2 * v_1_0_m1 + v_1_0_0 * v_1_0_1) + (v_m2_0_1 * v_m1_0_1 + v_m2_1_1 * v_m1_1_0 + v_m1_m1_2 * v_0_m1_1 + v_m1_0_0 * v_0_1_0 + v_m1_0_1 * v_0_0_m1 + v_m1_0_2 * v_0_0_1 + v_m1_1_0 * v_0_m1_1 + v_m1_2_0 * v_0_1_0 + v_0_m1_m1 * v_0_0_m1 + v_0_m1_0 * v_1_0_0 + v_0_m1_1 * v_1_m2_1 + v_0_0_m1 * v_0_1_0 + v_0_0_1 * v_0_1_1 + v_0_1_m1 * v_0_2_m1 + v_0_1_0 * v_0_2_m1 + v_1_m2_1 * v_1_m1_0 + v_1_0_m1 * v_1_1_m2 + v_1_0_0 * v_1_1_0)) + ((v_m2_1_0 * v_m1_0_0 + v_m1_m1_0 * v_m1_0_0 + v_m1_0_m1 * v_m1_0_0 + v_m1_0_0 * v_1_m1_0 + v_m1_0_1 * v_0_1_m1 + v_m1_1_0 * v_m1_2_m1 + v_m1_1_0 * v_1_0_m1 + v_0_m2_1 * v_0_m1_0 + v_0_m1_0 * v_0_0_1 + v_0_m1_1 * v_0_m1_2 + v_0_m1_1 * v_1_0_m1 + v_0_0_m1 * v_1_0_m2 + v_0_0_1 * v_1_0_m1 + v_0_1_m1 * v_1_m1_0 + v_0_1_0 * v_1_m1_0 + v_1_m1_0 * v_2_m1_m1 + v_1_0_m1 * v_2_m1_m1 + v_1_0_0 * v_2_m1_0) + (v_m2_1_0 * v_m1_1_0 + v_m1_m1_0 * v_0_m1_0 + v_m1_0_m1 * v_0_0_m1 + v_m1_0_0 * v_1_0_m1 + v_m1_0_1 * v_1_m1_0 + v_m1_1_0 * v_m1_2_0 + v_m1_1_0 * v_1_0_0 + v_0_m2_1 * v_0_m1_1 + v_0_m1_0 * v_0_1_m1 + v_0_m1_1 * v_0_0_m1 + v_0_m1_2 * v_0_0_1 + v_0_0_m1 * v_1_0_0 + v_0_0_1 * v_1_0_1 + v_0_1_m1 * v_1_1_m2 + v_0_1_0 * v_1_1_0 + v_1_m1_0 * v_2_m1_0 + v_1_0_m1 * v_2_0_m1 + v_1_0_0 * v_2_0_m1));
  F[8] = ((v_m1_0_0 * v_m1_0_1 * v_m1_1_0 + v_0_m1_0 * v_0_m1_1 * v_1_m1_0) + (v_m1_0_0 * v_0_m1_0 * v_0_0_m1 + v_0_0_m1 * v_0_1_m1 * v_1_0_m1)) + ((v_m1_0_1 * v_0_m1_1 * v_0_0_1 + v_0_0_1 * v_0_1_0 * v_1_0_0) + (v_m1_1_0 * v_0_1_m1 * v_0_1_0 + v_1_m1_0 * v_1_0_m1 * v_1_0_0));
}
// Byte-parallel features: ld(di,dj,dk) returns a word of four sites' occupants (one
// per byte); F[k] receives the four sites' local sums, one per byte.
template <class Loader>
__device__ __forceinline__ void features_quad(const Loader& ld, uint32_t (&F)[NFEAT]) {
  const uint32_t v_m2_0_0 = ld(-2, 0, 0);
  const uint32_t v_m2_0_1 = ld(-2, 0, 1);
  const uint32_t v_m2_0_2 = ld(-2, 0, 2);
  const uint32_t v_m2_1_0 = ld(-2, 1, 0);
  const uint32_t v_m2_1_1 = ld(-2, 1, 1);
  const uint32_t v_m2_2_0 = ld(-2, 2, 0);
  const uint32_t v_m1_m1_0 = ld(-1, -1, 0);
  const uint32_t v_m1_m1_1 = ld(-1, -1, 1);
  const uint32_t v_m1_m1_2 = ld(-1, -1, 2);
  const uint32_t v_m1_0_m1 = ld(-1, 0, -1);
  const uint32_t v_m1_0_0 = ld(-1, 0, 0);
  const uint32_t v_m1_0_1 = ld(-1, 0, 1);
  const uint32_t v_m1_0_2 = ld(-1, 0, 2);
  const uint32_t v_m1_1_m1 = ld(-1, 1, -1);
  const uint32_t v_m1_1_0 = ld(-1, 1, 0);
  const uint32_t v_m1_1_1 = ld(-1, 1, 1);
  const uint32_t v_m1_2_m1 = ld(-1, 2, -1);
  const uint32_t v_m1_2_0 = ld(-1, 2, 0);
  const uint32_t v_0_m2_0 = ld(0, -2, 0);
  const uint32_t v_0_m2_1 = ld(0, -2, 1);
  const uint32_t v_0_m2_2 = ld(0, -2, 2);
  const uint32_t v_0_m1_m1 = ld(0, -1, -1);
  const uint32_t v_0_m1_0 = ld(0, -1, 0);
  const uint32_t v_0_m1_1 = ld(0, -1, 1);
  const uint32_t v_0_m1_2 = ld(0, -1, 2);
  const uint32_t v_0_0_m2 = ld(0, 0, -2);
  const uint32_t v_0_0_m1 = ld(0, 0, -1);
  const uint32_t v_0_0_1 = ld(0, 0, 1);
  const uint32_t v_0_0_2 = ld(0, 0, 2);
  const uint32_t v_0_1_m2 = ld(0, 1, -2);
  const uint32_t v_0_1_m1 = ld(0, 1, -1);
  const uint32_t v_0_1_0 = ld(0, 1, 0);
  const uint32_t v_0_1_1 = ld(0, 1, 1);
  const uint32_t v_0_2_m2 = ld(0, 2, -2);
  const uint32_t v_0_2_m1 = ld(0, 2, -1);
  const uint32_t v_0_2_0 = ld(0, 2, 0);
  const uint32_t v_1_m2_0 = ld(1, -2, 0);
  const uint32_t v_1_m2_1 = ld(1, -2, 1);
  const uint32_t v_1_m1_m1 = ld(1, -1, -1);
  const uint32_t v_1_m1_0 = ld(1, -1, 0);
  const uint32_t v_1_m1_1 = ld(1, -1, 1);
  const uint32_t v_1_0_m2 = ld(1, 0, -2);
  const uint32_t v_1_0_m1 = ld(1, 0, -1);
  const uint32_t v_1_0_0 = ld(1, 0, 0);
  const uint32_t v_1_0_1 = ld(1, 0, 1);
  const uint32_t v_1_1_m2 = ld(1, 1, -2);
  const uint32_t v_1_1_m1 = ld(1, 1, -1);
  const uint32_t v_1_1_0 = ld(1, 1, 0);
  const uint32_t v_2_m2_0 = ld(2, -2, 0);
  const uint32_t v_2_m1_m1 = ld(2, -1, -1);
  const uint32_t v_2_m1_0 = ld(2, -1, 0);
  const uint32_t v_2_0_m2 = ld(2, 0, -2);
  const uint32_t v_2_0_m1 = ld(2, 0, -1);
  const uint32_t v_2_0_0 = ld(2, 0, 0);
  const uint32_t m_v_0_0_1 = v_0_0_1 * 0xFFu;
  const uint32_t m_v_0_0_m1 = v_0_0_m1 * 0xFFu;
  const uint32_t m_v_0_1_0 = v_0_1_0 * 0xFFu;
  const uint32_t m_v_0_1_m1 = v_0_1_m1 * 0xFFu;
  const uint32_t m_v_0_m1_0 = v_0_m1_0 * 0xFFu;
  const uint32_t m_v_0_m1_1 = v_0_m1_1 * 0xFFu;
  const uint32_t m_v_1_0_0 = v_1_0_0 * 0xFFu;
  const uint32_t m_v_1_0_m1 = v_1_0_m1 * 0xFFu;
  const uint32_t m_v_1_m1_0 = v_1_m1_0 * 0xFFu;
  const uint32_t m_v_m1_0_0 = v_m1_0_0 * 0xFFu;
  const uint32_t m_v_m1_0_1 = v_m1_0_1 * 0xFFu;
  const uint32_t m_v_m1_1_0 = v_m1_1_0 * 0xFFu;
  F[0] = 1u * 0x01010101u;
  F[1] = ((v_m1_0_0 + v_0_m1_1 + v_0_1_0) + (v_m1_0_1 + v_0_0_m1 + v_1_m1_0)) + ((v_m1_1_0 + v_0_0_1 + v_1_0_m1) + (v_0_m1_0 + v_0_1_m1 + v_1_0_0));
  F[2] = ((v_m1_m1_1 + v_1_m1_1) + (v_m1_1_m1 + v_1_1_m1)) + ((v_m1_1_1) + (v_1_m1_m1));
  F[3] = ((v_m2_0_1 + v_m1_m1_2 + v_m1_2_0 + v_0_1_m2 + v_1_m2_1 + v_1_1_0) + (v_m2_1_0 + v_m1_0_m1 + v_0_m2_1 + v_0_1_1 + v_1_0_m2 + v_2_m1_m1)) + ((v_m2_1_1 + v_m1_0_2 + v_0_m1_m1 + v_0_2_m1 + v_1_0_1 + v_2_m1_0) + (v_m1_m1_0 + v_m1_2_m1 + v_0_m1_2 + v_1_m2_0 + v_1_1_m2 + v_2_0_m1));
  F[4] = ((v_m2_0_0 + v_0_m2_2 + v_0_2_0) + (v_m2_0_2 + v_0_0_m2 + v_2_m2_0)) + ((v_m2_2_0 + v_0_0_2 + v_2_0_m2) + (v_0_m2_0 + v_0_2_m2 + v_2_0_0));
  F[5] = (((m_v_0_0_1 & (v_m1_0_1 + v_0_m1_1 + v_0_1_0 + v_1_0_0)) + (v_m1_0_0 & v_m1_0_1) + (v_0_1_m1 & v_0_1_0)) + ((m_v_0_0_m1 & (v_m1_0_0 + v_0_m1_0 + v_0_1_m1 + v_1_0_m1)) + (v_m1_0_0 & v_0_m1_0) + (v_0_1_m1 & v_1_0_m1))) + (((m_v_1_m1_0 & (v_0_m1_0 + v_0_m1_1 + v_1_0_m1 + v_1_0_0)) + (v_m1_0_1 & v_0_m1_1) + (v_0_1_0 & v_1_0_0)) + ((m_v_m1_1_0 & (v_m1_0_0 + v_m1_0_1 + v_0_1_m1 + v_0_1_0)) + (v_0_m1_0 & v_0_m1_1) + (v_1_0_m1 & v_1_0_0)));
  F[6] = (((m_v_0_0_1 & (v_m1_1_0 + v_m1_1_1 + v_1_m1_0 + v_1_m1_1)) + (m_v_0_m1_0 & (v_m1_m1_1 + v_m1_0_1 + v_1_m1_m1 + v_1_0_m1)) + (v_m1_0_0 & v_m1_1_m1) + (v_1_m1_m1 & v_1_m1_0) + (v_1_0_m1 & v_1_1_m1)) + ((m_v_0_0_m1 & (v_m1_1_m1 + v_m1_1_0 + v_1_m1_m1 + v_1_m1_0)) + (m_v_0_m1_1 & (v_m1_m1_1 + v_m1_0_0 + v_1_m1_1 + v_1_0_0)) + (v_m1_0_1 & v_m1_1_1) + (v_1_m1_m1 & v_1_0_m1) + (v_1_0_0 & v_1_1_m1))) + (((m_v_0_1_0 & (v_m1_0_1 + v_m1_1_1 + v_1_0_m1 + v_1_1_m1)) + (v_m1_m1_1 & v_m1_0_0) + (v_m1_1_m1 & v_m1_1_0) + (v_1_m1_0 & v_1_m1_1)) + ((m_v_0_1_m1 & (v_m1_0_0 + v_m1_1_m1 + v_1_0_0 + v_1_1_m1)) + (v_m1_m1_1 & v_m1_0_1) + (v_m1_1_0 & v_m1_1_1) + (v_1_m1_1 & v_1_0_0)));
  F[7] = (((m_v_0_0_1 & (v_m1_0_0 + v_m1_0_2 + v_0_m1_0 + v_0_m1_2 + v_0_1_m1 + v_0_1_1 + v_1_0_m1 + v_1_0_1)) + (m_v_0_1_0 & (v_m1_0_0 + v_m1_2_0 + v_0_m1_1 + v_0_1_1 + v_0_2_m1 + v_1_1_0)) + (m_v_0_m1_0 & (v_m1_m1_0 + v_0_m2_1 + v_0_m1_m1 + v_1_m2_0))) + ((m_v_0_0_m1 & (v_m1_0_m1 + v_m1_0_1 + v_0_m1_m1 + v_0_m1_1 + v_0_1_m2 + v_0_1_0 + v_1_0_m2 + v_1_0_0)) + (m_v_0_1_m1 & (v_m1_0_1 + v_m1_2_m1 + v_0_m1_0 + v_0_1_m2 + v_0_2_m1 + v_1_1_m2)) + (m_v_0_m1_1 & (v_m1_m1_2 + v_0_m2_1 + v_0_m1_2 + v_1_m2_1)))) + (((m_v_1_m1_0 & (v_m1_0_0 + v_m1_0_1 + v_0_1_m1 + v_0_1_0 + v_1_m2_0 + v_1_m2_1 + v_2_m1_m1 + v_2_m1_0)) + (m_v_1_0_0 & (v_m1_0_1 + v_0_m1_0 + v_1_0_1 + v_1_1_0 + v_2_m1_0 + v_2_0_m1)) + (m_v_m1_0_0 & (v_m2_0_1 + v_m2_1_0 + v_m1_m1_0 + v_m1_0_m1))) + ((m_v_m1_1_0 & (v_m2_1_0 + v_m2_1_1 + v_m1_2_m1 + v_m1_2_0 + v_0_m1_0 + v_0_m1_1 + v_1_0_m1 + v_1_0_0)) + (m_v_1_0_m1 & (v_m1_0_0 + v_0_m1_1 + v_1_0_m2 + v_1_1_m2 + v_2_m1_m1 + v_2_0_m1)) + (m_v_m1_0_1 & (v_m2_0_1 + v_m2_1_1 + v_m1_m1_2 + v_m1_0_2))));
  F[8] = (((v_m1_0_0 & v_m1_0_1 & v_m1_1_0) + (v_0_m1_0 & v_0_m1_1 & v_1_m1_0)) + ((v_m1_0_0 & v_0_m1_0 & v_0_0_m1) + (v_0_0_m1 & v_0_1_m1 & v_1_0_m1))) + (((v_m1_0_1 & v_0_m1_1 & v_0_0_1) + (v_0_0_1 & v_0_1_0 & v_1_0_0)) + ((v_m1_1_0 & v_0_1_m1 & v_0_1_0) + (v_1_m1_0 & v_1_0_m1 & v_1_0_0)));
}
// ---- word-layout pipelines (early / late split of features_quad)
constexpr int NPIPE = 2;
__host__ __device__ constexpr int pipe_colouring(int p, int q) {
  constexpr int t[NPIPE * 4] = {4, 5, 14, 16, 4, 6, 15, 16};
  return t[p * 4 + q];  // a, b, c, m
}
template <int P>
struct Pipe;
// colouring (4 i + 5 j + 14 k) mod 16: late neighbours (-1, 1, 1), (1, -1, 0)
template <>
struct Pipe<0> {
  static constexpr int NKEEP = 5;
  // late groups g (AND of late neighbours); F[k] gains sum over terms (g, k, keep, n) of
  // n * group_g * (keep < 0 ? 1 : K[keep]) per byte
  static constexpr int NGROUP = 2;
  static constexpr int NTERM = 7;
  __host__ __device__ static constexpr int term_group(int i) {
    constexpr int t[NTERM] = {0, 1, 0, 0, 1, 0, 0};
    return t[i];
  }
  __host__ __device__ static constexpr int term_feature(int i) {
    constexpr int t[NTERM] = {1, 2, 5, 6, 6, 7, 8};
    return t[i];
  }
  __host__ __device__ static constexpr int term_keep(int i) {
    constexpr int t[NTERM] = {-1, -1, 0, 1, 2, 3, 4};
    return t[i];
  }
  __host__ __device__ static constexpr int term_count(int i) {
    constexpr int t[NTERM] = {1, 1, 1, 1, 1, 1, 1};
    return t[i];
  }
  struct State {
    uint32_t E[NFEAT];
    uint32_t K[NKEEP];
    uint32_t own;
  };
  template <class Loader>
  __device__ static __forceinline__ void early(const Loader& ld, State& s) {
    const uint32_t v_m2_0_0 = ld(-2, 0, 0);
    const uint32_t v_m2_0_1 = ld(-2, 0, 1);
    const uint32_t v_m2_0_2 = ld(-2, 0, 2);
    const uint32_t v_m2_1_0 = ld(-2, 1, 0);
    const uint32_t v_m2_1_1 = ld(-2, 1, 1);
    const uint32_t v_m2_2_0 = ld(-2, 2, 0);
    const uint32_t v_m1_m1_0 = ld(-1, -1, 0);
    const uint32_t v_m1_m1_1 = ld(-1, -1, 1);
    const uint32_t v_m1_m1_2 = ld(-1, -1, 2);
    const uint32_t v_m1_0_m1 = ld(-1, 0, -1);
    const uint32_t v_m1_0_0 = ld(-1, 0, 0);
    const uint32_t v_m1_0_1 = ld(-1, 0, 1);
    const uint32_t v_m1_0_2 = ld(-1, 0, 2);
    const uint32_t v_m1_1_m1 = ld(-1, 1, -1);
    const uint32_t v_m1_1_0 = ld(-1, 1, 0);
    const uint32_t v_m1_2_m1 = ld(-1, 2, -1);
    const uint32_t v_m1_2_0 = ld(-1, 2, 0);
    const uint32_t v_0_m2_0 = ld(0, -2, 0);
    const uint32_t v_0_m2_1 = ld(0, -2, 1);
    const uint32_t v_0_m2_2 = ld(0, -2, 2);
    const uint32_t v_0_m1_m1 = ld(0, -1, -1);
    const uint32_t v_0_m1_0 = ld(0, -1, 0);
    const uint32_t v_0_m1_1 = ld(0, -1, 1);
    const uint32_t v_0_m1_2 = ld(0, -1, 2);
    const uint32_t v_0_0_m2 = ld(0, 0, -2);
    const uint32_t v_0_0_m1 = ld(0, 0, -1);
    const uint32_t v_0_0_1 = ld(0, 0, 1);
    const uint32_t v_0_0_2 = ld(0, 0, 2);
    const uint32_t v_0_1_m2 = ld(0, 1, -2);
    const uint32_t v_0_1_m1 = ld(0, 1, -1);
    const uint32_t v_0_1_0 = ld(0, 1, 0);
    const uint32_t v_0_1_1 = ld(0, 1, 1);
    const uint32_t v_0_2_m2 = ld(0, 2, -2);
    const uint32_t v_0_2_m1 = ld(0, 2, -1);
    const uint32_t v_0_2_0 = ld(0, 2, 0);
    const uint32_t v_1_m2_0 = ld(1, -2, 0);
    const uint32_t v_1_m2_1 = ld(1, -2, 1);
    const uint32_t v_1_m1_m1 = ld(1, -1, -1);
    const uint32_t v_1_m1_1 = ld(1, -1, 1);
    const uint32_t v_1_0_m2 = ld(1, 0, -2);
    const uint32_t v_1_0_m1 = ld(1, 0, -1);
    const uint32_t v_1_0_0 = ld(1, 0, 0);
    const uint32_t v_1_0_1 = ld(1, 0, 1);
    const uint32_t v_1_1_m2 = ld(1, 1, -2);
    const uint32_t v_1_1_m1 = ld(1, 1, -1);
    const uint32_t v_1_1_0 = ld(1, 1, 0);
    const uint32_t v_2_m2_0 = ld(2, -2, 0);
    const uint32_t v_2_m1_m1 = ld(2, -1, -1);
    const uint32_t v_2_m1_0 = ld(2, -1, 0);
    const uint32_t v_2_0_m2 = ld(2, 0, -2);
    const uint32_t v_2_0_m1 = ld(2, 0, -1);
    const uint32_t v_2_0_0 = ld(2, 0, 0);
    s.own = ld(0, 0, 0);
    const uint32_t m_v_0_0_1 = v_0_0_1 * 0xFFu;
    const uint32_t m_v_0_0_m1 = v_0_0_m1 * 0xFFu;
    const uint32_t m_v_0_1_0 = v_0_1_0 * 0xFFu;
    const uint32_t m_v_0_1_m1 = v_0_1_m1 * 0xFFu;
    const uint32_t m_v_0_m1_0 = v_0_m1_0 * 0xFFu;
    const uint32_t m_v_0_m1_1 = v_0_m1_1 * 0xFFu;
    const uint32_t m_v_1_0_0 = v_1_0_0 * 0xFFu;
    const uint32_t m_v_1_0_m1 = v_1_0_m1 * 0xFFu;
    const uint32_t m_v_m1_0_0 = v_m1_0_0 * 0xFFu;
    const uint32_t m_v_m1_0_1 = v_m1_0_1 * 0xFFu;
    const uint32_t m_v_m1_1_0 = v_m1_1_0 * 0xFFu;
    s.E[0] = 1u * 0x01010101u;
    s.E[1] = ((v_m1_0_0 + v_0_m1_1 + v_0_1_0) + (v_m1_0_1 + v_0_0_m1 + v_1_0_m1)) + ((v_m1_1_0 + v_0_0_1 + v_1_0_0) + (v_0_m1_0 + v_0_1_m1));
    s.E[2] = ((v_m1_m1_1 + v_1_1_m1) + (v_m1_1_m1)) + ((v_1_m1_m1) + (v_1_m1_1));
    s.E[3] = ((v_m2_0_1 + v_m1_m1_2 + v_m1_2_0 + v_0_1_m2 + v_1_m2_1 + v_1_1_0) + (v_m2_1_0 + v_m1_0_m1 + v_0_m2_1 + v_0_1_1 + v_1_0_m2 + v_2_m1_m1)) + ((v_m2_1_1 + v_m1_0_2 + v_0_m1_m1 + v_0_2_m1 + v_1_0_1 + v_2_m1_0) + (v_m1_m1_0 + v_m1_2_m1 + v_0_m1_2 + v_1_m2_0 + v_1_1_m2 + v_2_0_m1));
    s.E[4] = ((v_m2_0_0 + v_0_m2_2 + v_0_2_0) + (v_m2_0_2 + v_0_0_m2 + v_2_m2_0)) + ((v_m2_2_0 + v_0_0_2 + v_2_0_m2) + (v_0_m2_0 + v_0_2_m2 + v_2_0_0));
    s.E[5] = (((m_v_0_0_1 & (v_m1_0_1 + v_0_m1_1 + v_0_1_0 + v_1_0_0)) + (m_v_0_m1_0 & (v_m1_0_0 + v_0_m1_1))) + ((m_v_0_0_m1 & (v_m1_0_0 + v_0_m1_0 + v_0_1_m1 + v_1_0_m1)) + (m_v_1_0_m1 & (v_0_1_m1 + v_1_0_0)))) + (((m_v_m1_1_0 & (v_m1_0_0 + v_m1_0_1 + v_0_1_m1 + v_0_1_0)) + (m_v_m1_0_1 & (v_m1_0_0 + v_0_m1_1))) + ((m_v_0_1_0 & (v_0_1_m1 + v_1_0_0))));
    s.E[6] = (((m_v_0_1_m1 & (v_m1_0_0 + v_m1_1_m1 + v_1_0_0 + v_1_1_m1)) + (m_v_0_1_0 & (v_m1_0_1 + v_1_0_m1 + v_1_1_m1)) + (m_v_m1_0_0 & (v_m1_m1_1 + v_m1_1_m1))) + ((m_v_0_m1_0 & (v_m1_m1_1 + v_m1_0_1 + v_1_m1_m1 + v_1_0_m1)) + (m_v_0_0_1 & (v_m1_1_0 + v_1_m1_1)) + (v_m1_m1_1 & v_m1_0_1))) + (((m_v_0_m1_1 & (v_m1_m1_1 + v_m1_0_0 + v_1_m1_1 + v_1_0_0)) + (m_v_1_0_0 & (v_1_m1_1 + v_1_1_m1)) + (v_m1_1_m1 & v_m1_1_0)) + ((m_v_0_0_m1 & (v_m1_1_m1 + v_m1_1_0 + v_1_m1_m1)) + (m_v_1_0_m1 & (v_1_m1_m1 + v_1_1_m1))));
    s.E[7] = (((m_v_0_0_1 & (v_m1_0_0 + v_m1_0_2 + v_0_m1_0 + v_0_m1_2 + v_0_1_m1 + v_0_1_1 + v_1_0_m1 + v_1_0_1)) + (m_v_0_1_m1 & (v_m1_0_1 + v_m1_2_m1 + v_0_m1_0 + v_0_1_m2 + v_0_2_m1 + v_1_1_m2)) + (m_v_0_m1_1 & (v_m1_m1_2 + v_0_m2_1 + v_0_m1_2 + v_1_m2_1))) + ((m_v_0_0_m1 & (v_m1_0_m1 + v_m1_0_1 + v_0_m1_m1 + v_0_m1_1 + v_0_1_m2 + v_0_1_0 + v_1_0_m2 + v_1_0_0)) + (m_v_1_0_0 & (v_m1_0_1 + v_0_m1_0 + v_1_0_1 + v_1_1_0 + v_2_m1_0 + v_2_0_m1)) + (m_v_m1_0_0 & (v_m2_0_1 + v_m2_1_0 + v_m1_m1_0 + v_m1_0_m1)))) + (((m_v_m1_1_0 & (v_m2_1_0 + v_m2_1_1 + v_m1_2_m1 + v_m1_2_0 + v_0_m1_0 + v_0_m1_1 + v_1_0_m1 + v_1_0_0)) + (m_v_1_0_m1 & (v_m1_0_0 + v_0_m1_1 + v_1_0_m2 + v_1_1_m2 + v_2_m1_m1 + v_2_0_m1)) + (m_v_m1_0_1 & (v_m2_0_1 + v_m2_1_1 + v_m1_m1_2 + v_m1_0_2))) + ((m_v_0_1_0 & (v_m1_0_0 + v_m1_2_0 + v_0_m1_1 + v_0_1_1 + v_0_2_m1 + v_1_1_0)) + (m_v_0_m1_0 & (v_m1_m1_0 + v_0_m2_1 + v_0_m1_m1 + v_1_m2_0))));
    s.E[8] = (((v_m1_0_0 & v_m1_0_1 & v_m1_1_0) + (v_0_0_m1 & v_0_1_m1 & v_1_0_m1)) + ((v_m1_0_0 & v_0_m1_0 & v_0_0_m1) + (v_0_0_1 & v_0_1_0 & v_1_0_0))) + (((v_m1_0_1 & v_0_m1_1 & v_0_0_1)) + ((v_m1_1_0 & v_0_1_m1 & v_0_1_0)));
    s.K[0] = v_0_m1_0 + v_0_m1_1 + v_1_0_m1 + v_1_0_0;
    s.K[1] = v_0_0_m1 + v_0_0_1 + v_1_m1_m1 + v_1_m1_1;
    s.K[2] = v_m1_0_1 + v_m1_1_0 + v_0_0_1 + v_0_1_0;
    s.K[3] = v_m1_0_0 + v_m1_0_1 + v_0_1_m1 + v_0_1_0 + v_1_m2_0 + v_1_m2_1 + v_2_m1_m1 + v_2_m1_0;
    s.K[4] = (v_0_m1_0 & v_0_m1_1) + (v_1_0_m1 & v_1_0_0);
  }
  template <class Loader>
  __device__ static __forceinline__ void late(const Loader& ld, const State& s, uint32_t (&F)[NFEAT],
                                              uint32_t (&Lw)[NGROUP]) {
    const uint32_t v_m1_1_1 = ld(-1, 1, 1);
    const uint32_t v_1_m1_0 = ld(1, -1, 0);
    F[0] = s.E[0];
    F[1] = s.E[1] + v_1_m1_0;
    F[2] = s.E[2] + v_m1_1_1;
    F[3] = s.E[3];
    F[4] = s.E[4];
    F[5] = s.E[5] + (((v_1_m1_0) * 0xFFu) & s.K[0]);
    F[6] = s.E[6] + (((v_1_m1_0) * 0xFFu) & s.K[1]) + (((v_m1_1_1) * 0xFFu) & s.K[2]);
    F[7] = s.E[7] + (((v_1_m1_0) * 0xFFu) & s.K[3]);
    F[8] = s.E[8] + (((v_1_m1_0) * 0xFFu) & s.K[4]);
    Lw[0] = v_1_m1_0;
    Lw[1] = v_m1_1_1;
  }
};
// colouring (4 i + 6 j + 15 k) mod 16: late neighbours (0, 0, 1), (1, -1, -1)
template <>
struct Pipe<1> {
  static constexpr int NKEEP = 5;
  // late groups g (AND of late neighbours); F[k] gains sum over terms (g, k, keep, n) of
  // n * group_g * (keep < 0 ? 1 : K[keep]) per byte
  static constexpr int NGROUP = 2;
  static constexpr int NTERM = 7;
  __host__ __device__ static constexpr int term_group(int i) {
    constexpr int t[NTERM] = {0, 1, 0, 0, 1, 0, 0};
    return t[i];
  }
  __host__ __device__ static constexpr int term_feature(int i) {
    constexpr int t[NTERM] = {1, 2, 5, 6, 6, 7, 8};
    return t[i];
  }
  __host__ __device__ static constexpr int term_keep(int i) {
    constexpr int t[NTERM] = {-1, -1, 0, 1, 2, 3, 4};
    return t[i];
  }
  __host__ __device__ static constexpr int term_count(int i) {
    constexpr int t[NTERM] = {1, 1, 1, 1, 1, 1, 1};
    return t[i];
  }
  struct State {
    uint32_t E[NFEAT];
    uint32_t K[NKEEP];
    uint32_t own;
  };
  template <class Loader>
  __device__ static __forceinline__ void early(const Loader& ld, State& s) {
    const uint32_t v_m2_0_0 = ld(-2, 0, 0);
    const uint32_t v_m2_0_1 = ld(-2, 0, 1);
    const uint32_t v_m2_0_2 = ld(-2, 0, 2);
    const uint32_t v_m2_1_0 = ld(-2, 1, 0);
    const uint32_t v_m2_1_1 = ld(-2, 1, 1);
    const uint32_t v_m2_2_0 = ld(-2, 2, 0);
    const uint32_t v_m1_m1_0 = ld(-1, -1, 0);
    const uint32_t v_m1_m1_1 = ld(-1, -1, 1);
    const uint32_t v_m1_m1_2 = ld(-1, -1, 2);
    const uint32_t v_m1_0_m1 = ld(-1, 0, -1);
    const uint32_t v_m1_0_0 = ld(-1, 0, 0);
    const uint32_t v_m1_0_1 = ld(-1, 0, 1);
    const uint32_t v_m1_0_2 = ld(-1, 0, 2);
    const uint32_t v_m1_1_m1 = ld(-1, 1, -1);
    const uint32_t v_m1_1_0 = ld(-1, 1, 0);
    const uint32_t v_m1_1_1 = ld(-1, 1, 1);
    const uint32_t v_m1_2_m1 = ld(-1, 2, -1);
    const uint32_t v_m1_2_0 = ld(-1, 2, 0);
    const uint32_t v_0_m2_0 = ld(0, -2, 0);
    const uint32_t v_0_m2_1 = ld(0, -2, 1);
    const uint32_t v_0_m2_2 = ld(0, -2, 2);
    const uint32_t v_0_m1_m1 = ld(0, -1, -1);
    const uint32_t v_0_m1_0 = ld(0, -1, 0);
    const uint32_t v_0_m1_1 = ld(0, -1, 1);
    const uint32_t v_0_m1_2 = ld(0, -1, 2);
    const uint32_t v_0_0_m2 = ld(0, 0, -2);
    const uint32_t v_0_0_m1 = ld(0, 0, -1);
    const uint32_t v_0_0_2 = ld(0, 0, 2);
    const uint32_t v_0_1_m2 = ld(0, 1, -2);
    const uint32_t v_0_1_m1 = ld(0, 1, -1);
    const uint32_t v_0_1_0 = ld(0, 1, 0);
    const uint32_t v_0_1_1 = ld(0, 1, 1);
    const uint32_t v_0_2_m2 = ld(0, 2, -2);
    const uint32_t v_0_2_m1 = ld(0, 2, -1);
    const uint32_t v_0_2_0 = ld(0, 2, 0);
    const uint32_t v_1_m2_0 = ld(1, -2, 0);
    const uint32_t v_1_m2_1 = ld(1, -2, 1);
    const uint32_t v_1_m1_0 = ld(1, -1, 0);
    const uint32_t v_1_m1_1 = ld(1, -1, 1);
    const uint32_t v_1_0_m2 = ld(1, 0, -2);
    const uint32_t v_1_0_m1 = ld(1, 0, -1);
    const uint32_t v_1_0_0 = ld(1, 0, 0);
    const uint32_t v_1_0_1 = ld(1, 0, 1);
    const uint32_t v_1_1_m2 = ld(1, 1, -2);
    const uint32_t v_1_1_m1 = ld(1, 1, -1);
    const uint32_t v_1_1_0 = ld(1, 1, 0);
    const uint32_t v_2_m2_0 = ld(2, -2, 0);
    const uint32_t v_2_m1_m1 = ld(2, -1, -1);
    const uint32_t v_2_m1_0 = ld(2, -1, 0);
    const uint32_t v_2_0_m2 = ld(2, 0, -2);
    const uint32_t v_2_0_m1 = ld(2, 0, -1);
    const uint32_t v_2_0_0 = ld(2, 0, 0);
    s.own = ld(0, 0, 0);
    const uint32_t m_v_0_0_m1 = v_0_0_m1 * 0xFFu;
    const uint32_t m_v_0_1_0 = v_0_1_0 * 0xFFu;
    const uint32_t m_v_0_1_m1 = v_0_1_m1 * 0xFFu;
    const uint32_t m_v_0_m1_0 = v_0_m1_0 * 0xFFu;
    const uint32_t m_v_0_m1_1 = v_0_m1_1 * 0xFFu;
    const uint32_t m_v_1_0_0 = v_1_0_0 * 0xFFu;
    const uint32_t m_v_1_0_m1 = v_1_0_m1 * 0xFFu;
    const uint32_t m_v_1_m1_0 = v_1_m1_0 * 0xFFu;
    const uint32_t m_v_m1_0_0 = v_m1_0_0 * 0xFFu;
    const uint32_t m_v_m1_0_1 = v_m1_0_1 * 0xFFu;
    const uint32_t m_v_m1_1_0 = v_m1_1_0 * 0xFFu;
    s.E[0] = 1u * 0x01010101u;
    s.E[1] = ((v_m1_0_0 + v_0_m1_1 + v_1_m1_0) + (v_m1_0_1 + v_0_0_m1 + v_1_0_m1)) + ((v_m1_1_0 + v_0_1_m1 + v_1_0_0) + (v_0_m1_0 + v_0_1_0));
    s.E[2] = ((v_m1_m1_1 + v_1_1_m1) + (v_m1_1_m1)) + ((v_m1_1_1) + (v_1_m1_1));
    s.E[3] = ((v_m2_0_1 + v_m1_m1_2 + v_m1_2_0 + v_0_1_m2 + v_1_m2_1 + v_1_1_0) + (v_m2_1_0 + v_m1_0_m1 + v_0_m2_1 + v_0_1_1 + v_1_0_m2 + v_2_m1_m1)) + ((v_m2_1_1 + v_m1_0_2 + v_0_m1_m1 + v_0_2_m1 + v_1_0_1 + v_2_m1_0) + (v_m1_m1_0 + v_m1_2_m1 + v_0_m1_2 + v_1_m2_0 + v_1_1_m2 + v_2_0_m1));
    s.E[4] = ((v_m2_0_0 + v_0_m2_2 + v_0_2_0) + (v_m2_0_2 + v_0_0_m2 + v_2_m2_0)) + ((v_m2_2_0 + v_0_0_2 + v_2_0_m2) + (v_0_m2_0 + v_0_2_m2 + v_2_0_0));
    s.E[5] = (((m_v_0_0_m1 & (v_m1_0_0 + v_0_m1_0 + v_0_1_m1 + v_1_0_m1)) + (m_v_0_m1_0 & (v_m1_0_0 + v_0_m1_1))) + ((m_v_1_m1_0 & (v_0_m1_0 + v_0_m1_1 + v_1_0_m1 + v_1_0_0)) + (m_v_1_0_m1 & (v_0_1_m1 + v_1_0_0)))) + (((m_v_m1_1_0 & (v_m1_0_0 + v_m1_0_1 + v_0_1_m1 + v_0_1_0)) + (m_v_m1_0_1 & (v_m1_0_0 + v_0_m1_1))) + ((m_v_0_1_0 & (v_0_1_m1 + v_1_0_0))));
    s.E[6] = (((m_v_0_1_0 & (v_m1_0_1 + v_m1_1_1 + v_1_0_m1 + v_1_1_m1)) + (m_v_0_m1_0 & (v_m1_m1_1 + v_m1_0_1 + v_1_0_m1)) + (m_v_m1_1_0 & (v_m1_1_m1 + v_m1_1_1))) + ((m_v_0_1_m1 & (v_m1_0_0 + v_m1_1_m1 + v_1_0_0 + v_1_1_m1)) + (m_v_1_0_0 & (v_1_m1_1 + v_1_1_m1)) + (v_1_m1_0 & v_1_m1_1))) + (((m_v_0_m1_1 & (v_m1_m1_1 + v_m1_0_0 + v_1_m1_1 + v_1_0_0)) + (m_v_m1_0_0 & (v_m1_m1_1 + v_m1_1_m1)) + (v_1_0_m1 & v_1_1_m1)) + ((m_v_0_0_m1 & (v_m1_1_m1 + v_m1_1_0 + v_1_m1_0)) + (m_v_m1_0_1 & (v_m1_m1_1 + v_m1_1_1))));
    s.E[7] = (((m_v_0_0_m1 & (v_m1_0_m1 + v_m1_0_1 + v_0_m1_m1 + v_0_m1_1 + v_0_1_m2 + v_0_1_0 + v_1_0_m2 + v_1_0_0)) + (m_v_0_1_m1 & (v_m1_0_1 + v_m1_2_m1 + v_0_m1_0 + v_0_1_m2 + v_0_2_m1 + v_1_1_m2)) + (m_v_0_m1_1 & (v_m1_m1_2 + v_0_m2_1 + v_0_m1_2 + v_1_m2_1))) + ((m_v_1_m1_0 & (v_m1_0_0 + v_m1_0_1 + v_0_1_m1 + v_0_1_0 + v_1_m2_0 + v_1_m2_1 + v_2_m1_m1 + v_2_m1_0)) + (m_v_1_0_0 & (v_m1_0_1 + v_0_m1_0 + v_1_0_1 + v_1_1_0 + v_2_m1_0 + v_2_0_m1)) + (m_v_m1_0_0 & (v_m2_0_1 + v_m2_1_0 + v_m1_m1_0 + v_m1_0_m1)))) + (((m_v_m1_1_0 & (v_m2_1_0 + v_m2_1_1 + v_m1_2_m1 + v_m1_2_0 + v_0_m1_0 + v_0_m1_1 + v_1_0_m1 + v_1_0_0)) + (m_v_1_0_m1 & (v_m1_0_0 + v_0_m1_1 + v_1_0_m2 + v_1_1_m2 + v_2_m1_m1 + v_2_0_m1)) + (m_v_m1_0_1 & (v_m2_0_1 + v_m2_1_1 + v_m1_m1_2 + v_m1_0_2))) + ((m_v_0_1_0 & (v_m1_0_0 + v_m1_2_0 + v_0_m1_1 + v_0_1_1 + v_0_2_m1 + v_1_1_0)) + (m_v_0_m1_0 & (v_m1_m1_0 + v_0_m2_1 + v_0_m1_m1 + v_1_m2_0))));
    s.E[8] = (((v_m1_0_0 & v_m1_0_1 & v_m1_1_0) + (v_0_0_m1 & v_0_1_m1 & v_1_0_m1)) + ((v_m1_0_0 & v_0_m1_0 & v_0_0_m1) + (v_1_m1_0 & v_1_0_m1 & v_1_0_0))) + (((v_m1_1_0 & v_0_1_m1 & v_0_1_0)) + ((v_0_m1_0 & v_0_m1_1 & v_1_m1_0)));
    s.K[0] = v_m1_0_1 + v_0_m1_1 + v_0_1_0 + v_1_0_0;
    s.K[1] = v_m1_1_0 + v_m1_1_1 + v_1_m1_0 + v_1_m1_1;
    s.K[2] = v_0_m1_0 + v_0_0_m1 + v_1_m1_0 + v_1_0_m1;
    s.K[3] = v_m1_0_0 + v_m1_0_2 + v_0_m1_0 + v_0_m1_2 + v_0_1_m1 + v_0_1_1 + v_1_0_m1 + v_1_0_1;
    s.K[4] = (v_m1_0_1 & v_0_m1_1) + (v_0_1_0 & v_1_0_0);
  }
  template <class Loader>
  __device__ static __forceinline__ void late(const Loader& ld, const State& s, uint32_t (&F)[NFEAT],
                                              uint32_t (&Lw)[NGROUP]) {
    const uint32_t v_0_0_1 = ld(0, 0, 1);
    const uint32_t v_1_m1_m1 = ld(1, -1, -1);
    F[0] = s.E[0];
    F[1] = s.E[1] + v_0_0_1;
    F[2] = s.E[2] + v_1_m1_m1;
    F[3] = s.E[3];
    F[4] = s.E[4];
    F[5] = s.E[5] + (((v_0_0_1) * 0xFFu) & s.K[0]);
    F[6] = s.E[6] + (((v_0_0_1) * 0xFFu) & s.K[1]) + (((v_1_m1_m1) * 0xFFu) & s.K[2]);
    F[7] = s.E[7] + (((v_0_0_1) * 0xFFu) & s.K[3]);
    F[8] = s.E[8] + (((v_0_0_1) * 0xFFu) & s.K[4]);
    Lw[0] = v_0_0_1;
    Lw[1] = v_1_m1_m1;
  }
};
// C[f] += sum over decorated clusters of class f anchored at this site (its
// lexicographically smallest member) of the product of integer psi values.
template <class Loader>
__device__ __forceinline__ void anchored(const Loader& ld, long long (&C)[NCLASS]) {
  const int v_m2_0_1 = ld(-2, 0, 1);
  const int v_m2_0_2 = ld(-2, 0, 2);
  const int v_m2_1_0 = ld(-2, 1, 0);
  const int v_m2_1_1 = ld(-2, 1, 1);
  const int v_m2_2_0 = ld(-2, 2, 0);
  const int v_m1_m1_2 = ld(-1, -1, 2);
  const int v_m1_0_1 = ld(-1, 0, 1);
  const int v_m1_0_2 = ld(-1, 0, 2);
  const int v_m1_1_0 = ld(-1, 1, 0);
  const int v_m1_1_1 = ld(-1, 1, 1);
  const int v_m1_2_m1 = ld(-1, 2, -1);
  const int v_m1_2_0 = ld(-1, 2, 0);
  const int v_0_m2_2 = ld(0, -2, 2);
  const int v_0_m1_1 = ld(0, -1, 1);
  const int v_0_m1_2 = ld(0, -1, 2);
  const int v_0_0_0 = ld(0, 0, 0);
  const int v_0_0_1 = ld(0, 0, 1);
  const int v_0_0_2 = ld(0, 0, 2);
  const int v_0_1_0 = ld(0, 1, 0);
  const int v_0_1_1 = ld(0, 1, 1);
  const int v_0_2_m1 = ld(0, 2, -1);
  const int v_0_2_0 = ld(0, 2, 0);
  const int v_1_m1_1 = ld(1, -1, 1);
  const int v_1_0_0 = ld(1, 0, 0);
  const int v_1_0_1 = ld(1, 0, 1);
  const int v_1_1_m1 = ld(1, 1, -1);
  const int v_1_1_0 = ld(1, 1, 0);
  const int v_2_0_0 = ld(2, 0, 0);
  C[0] += (long long)(1);
  C[1] += (long long)(v_0_0_0);
  C[2] += (long long)(((v_m1_0_1 * v_0_0_0 + v_0_0_0 * v_0_1_0) + (v_m1_1_0 * v_0_0_0 + v_0_0_0 * v_1_0_0)) + ((v_0_m1_1 * v_0_0_0) + (v_0_0_0 * v_0_0_1)));
  C[3] += (long long)(v_m1_1_1 * v_0_0_0 + v_0_0_0 * v_1_m1_1 + v_0_0_0 * v_1_1_m1);
  C[4] += (long long)(((v_m2_0_1 * v_0_0_0 + v_m1_0_2 * v_0_0_0 + v_0_0_0 * v_0_1_1) + (v_m2_1_0 * v_0_0_0 + v_m1_2_m1 * v_0_0_0 + v_0_0_0 * v_0_2_m1)) + ((v_m2_1_1 * v_0_0_0 + v_m1_2_0 * v_0_0_0 + v_0_0_0 * v_1_0_1) + (v_m1_m1_2 * v_0_0_0 + v_0_m1_2 * v_0_0_0 + v_0_0_0 * v_1_1_0)));
  C[5] += (long long)(((v_m2_0_2 * v_0_0_0 + v_0_0_0 * v_0_2_0) + (v_m2_2_0 * v_0_0_0 + v_0_0_0 * v_2_0_0)) + ((v_0_m2_2 * v_0_0_0) + (v_0_0_0 * v_0_0_2)));
  C[6] += (long long)(((v_m1_0_1 * v_m1_1_0 * v_0_0_0 + v_0_m1_1 * v_0_0_0 * v_0_0_1) + (v_m1_0_1 * v_0_m1_1 * v_0_0_0 + v_0_0_0 * v_0_0_1 * v_0_1_0)) + ((v_m1_0_1 * v_0_0_0 * v_0_0_1 + v_0_0_0 * v_0_0_1 * v_1_0_0) + (v_m1_1_0 * v_0_0_0 * v_0_1_0 + v_0_0_0 * v_0_1_0 * v_1_0_0)));
  C[7] += (long long)(((v_m1_0_1 * v_m1_1_1 * v_0_0_0 + v_m1_1_1 * v_0_0_0 * v_0_0_1 + v_0_0_0 * v_0_0_1 * v_1_m1_1) + (v_m1_0_1 * v_0_0_0 * v_0_1_0 + v_m1_1_1 * v_0_0_0 * v_0_1_0 + v_0_0_0 * v_0_1_0 * v_1_1_m1)) + ((v_m1_1_0 * v_m1_1_1 * v_0_0_0 + v_0_m1_1 * v_0_0_0 * v_1_m1_1 + v_0_0_0 * v_1_m1_1 * v_1_0_0) + (v_m1_1_0 * v_0_0_0 * v_0_0_1 + v_0_m1_1 * v_0_0_0 * v_1_0_0 + v_0_0_0 * v_1_0_0 * v_1_1_m1)));
  C[8] += (long long)(((v_m2_0_1 * v_m1_0_1 * v_0_0_0 + v_m1_m1_2 * v_m1_0_1 * v_0_0_0 + v_m1_0_2 * v_0_0_0 * v_0_0_1 + v_m1_1_0 * v_0_0_0 * v_1_0_0 + v_0_m1_2 * v_0_0_0 * v_0_0_1 + v_0_0_0 * v_0_1_0 * v_0_2_m1) + (v_m2_1_0 * v_m1_1_0 * v_0_0_0 + v_m1_m1_2 * v_0_m1_1 * v_0_0_0 + v_m1_1_0 * v_m1_2_m1 * v_0_0_0 + v_m1_2_0 * v_0_0_0 * v_0_1_0 + v_0_0_0 * v_0_0_1 * v_0_1_1 + v_0_0_0 * v_0_1_0 * v_1_1_0)) + ((v_m2_1_1 * v_m1_0_1 * v_0_0_0 + v_m1_0_1 * v_m1_0_2 * v_0_0_0 + v_m1_1_0 * v_m1_2_0 * v_0_0_0 + v_0_m1_1 * v_0_m1_2 * v_0_0_0 + v_0_0_0 * v_0_0_1 * v_1_0_1 + v_0_0_0 * v_1_0_0 * v_1_0_1) + (v_m2_1_1 * v_m1_1_0 * v_0_0_0 + v_m1_0_1 * v_0_0_0 * v_1_0_0 + v_m1_1_0 * v_0_m1_1 * v_0_0_0 + v_0_m1_1 * v_0_0_0 * v_0_1_0 + v_0_0_0 * v_0_1_0 * v_0_1_1 + v_0_0_0 * v_1_0_0 * v_1_1_0)));
  C[9] += (long long)(v_m1_0_1 * v_0_m1_1 * v_0_0_0 * v_0_0_1 + v_0_0_0 * v_0_0_1 * v_0_1_0 * v_1_0_0);
}
}}  // namespace

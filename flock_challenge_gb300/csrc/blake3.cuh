// BLAKE3 compression on the device, state held in registers.
//
// Follows the reference compression at
// crates/flock-prover/src/r1cs_hashes/blake3.rs:271-310 (IV, message
// permutation, column/diagonal G order, finalization XORs).
#pragma once
#include <cstdint>

namespace b3 {

__host__ __device__ constexpr uint32_t IV(int i) {
  return i == 0 ? 0x6a09e667u : i == 1 ? 0xbb67ae85u : i == 2 ? 0x3c6ef372u : i == 3 ? 0xa54ff53au
       : i == 4 ? 0x510e527fu : i == 5 ? 0x9b05688cu : i == 6 ? 0x1f83d9abu : 0x5be0cd19u;
}
enum : uint32_t { CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8 };

// Message words of the next round: m'[i] = m[PERM[i]] with the BLAKE3
// message permutation (2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8).
// Every index is a constant, so once the rounds are unrolled the permutation
// is register renaming and costs no instructions.
__device__ __forceinline__ void permute(uint32_t m[16]) {
  uint32_t t[16] = {m[2], m[6], m[3], m[10], m[7], m[0], m[4], m[13],
                    m[1], m[11], m[12], m[5], m[9], m[14], m[15], m[8]};
#pragma unroll
  for (int i = 0; i < 16; i++) m[i] = t[i];
}

__device__ __forceinline__ uint32_t rotr(uint32_t x, int n) { return __funnelshift_r(x, x, n); }

#define B3_G(a, b, c, d, mx, my)    \
  v[a] = v[a] + v[b] + (mx);        \
  v[d] = rotr(v[d] ^ v[a], 16);     \
  v[c] = v[c] + v[d];               \
  v[b] = rotr(v[b] ^ v[c], 12);     \
  v[a] = v[a] + v[b] + (my);        \
  v[d] = rotr(v[d] ^ v[a], 8);      \
  v[c] = v[c] + v[d];               \
  v[b] = rotr(v[b] ^ v[c], 7);

// Full compression; out[0..8] is the new chaining value, out[8..16] the
// second half of the extended output.
__device__ __forceinline__ void compress(const uint32_t cv[8], const uint32_t m[16], uint64_t counter,
                                         uint32_t block_len, uint32_t flags, uint32_t out[16]) {
  uint32_t v[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    IV(0), IV(1), IV(2), IV(3), (uint32_t)counter, (uint32_t)(counter >> 32), block_len, flags};
  uint32_t w[16];
#pragma unroll
  for (int i = 0; i < 16; i++) w[i] = m[i];
#pragma unroll
  for (int r = 0; r < 7; r++) {
    B3_G(0, 4, 8, 12, w[0], w[1]);
    B3_G(1, 5, 9, 13, w[2], w[3]);
    B3_G(2, 6, 10, 14, w[4], w[5]);
    B3_G(3, 7, 11, 15, w[6], w[7]);
    B3_G(0, 5, 10, 15, w[8], w[9]);
    B3_G(1, 6, 11, 12, w[10], w[11]);
    B3_G(2, 7, 8, 13, w[12], w[13]);
    B3_G(3, 4, 9, 14, w[14], w[15]);
    if (r < 6) permute(w);
  }
#pragma unroll
  for (int i = 0; i < 8; i++) {
    out[i] = v[i] ^ v[i + 8];
    out[i + 8] = v[i + 8] ^ cv[i];
  }
}

// Chaining-value-only compression with a zero counter (Merkle leaves/parents).
__device__ __forceinline__ void compress_cv(uint32_t cv[8], const uint32_t m[16], uint32_t block_len,
                                            uint32_t flags) {
  uint32_t v[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    IV(0), IV(1), IV(2), IV(3), 0u, 0u, block_len, flags};
  uint32_t w[16];
#pragma unroll
  for (int i = 0; i < 16; i++) w[i] = m[i];
#pragma unroll
  for (int r = 0; r < 7; r++) {
    B3_G(0, 4, 8, 12, w[0], w[1]);
    B3_G(1, 5, 9, 13, w[2], w[3]);
    B3_G(2, 6, 10, 14, w[4], w[5]);
    B3_G(3, 7, 11, 15, w[6], w[7]);
    B3_G(0, 5, 10, 15, w[8], w[9]);
    B3_G(1, 6, 11, 12, w[10], w[11]);
    B3_G(2, 7, 8, 13, w[12], w[13]);
    B3_G(3, 4, 9, 14, w[14], w[15]);
    if (r < 6) permute(w);
  }
#pragma unroll
  for (int i = 0; i < 8; i++) cv[i] = v[i] ^ v[i + 8];
}

}  // namespace b3

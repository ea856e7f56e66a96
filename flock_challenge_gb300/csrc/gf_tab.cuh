// Multiplication by a fixed GF(2^128) element through byte tables in shared
// memory. y -> t y is GF(2)-linear, so with T[(v << 4) + k] = t v x^(8k) (16
// byte positions k, 256 byte values v: 64 KiB) a product is the XOR of 16
// table entries, one per byte of y, with no carry-less multiply. Worth it when
// one CTA multiplies many elements by the same t (NTT twiddles of the upper
// layers, a sumcheck round's binding challenge). Slot (v << 4) + k lies in
// bank group k mod 8 and a thread visits the byte positions in an order
// XORed with its index mod 8, so eight consecutive threads read eight
// distinct bank groups: the random lookups are conflict-free.
#pragma once
#include "gf128.cuh"

constexpr int GF_TAB_ENTRIES = 16 * 256;      // slots of one byte-table set

// t * x^i for 0 <= i < 128: shift into 256 bits, then reduce.
__device__ __forceinline__ gf128 gf_mul_xpow_small(gf128 h, int i) {
  const uint64_t lo = h.w[0] | ((uint64_t)h.w[1] << 32), hi = h.w[2] | ((uint64_t)h.w[3] << 32);
  const int wsh = i >> 6, bsh = i & 63;
  const uint64_t s0 = lo << bsh, s1 = (hi << bsh) | (bsh ? lo >> (64 - bsh) : 0), s2 = bsh ? hi >> (64 - bsh) : 0;
  return wsh == 0 ? gf_reduce(s0, s1, s2, 0) : gf_reduce(0, s0, s1, s2);
}

__device__ __forceinline__ uint32_t gf_sel_word(const gf128& y, uint32_t j) {
  return (j & 2) ? ((j & 1) ? y.w[3] : y.w[2]) : ((j & 1) ? y.w[1] : y.w[0]);
}

// t * y from t's byte tables T. The thread visits byte position k = st ^ rot at
// step st (rot = thread index mod 8), so at every step eight consecutive
// threads read eight distinct bank groups (k mod 8 = (st mod 8) ^ rot). The
// bytes of y are permuted once to that order (a word swap for rot's bit 2, a
// byte permutation for its bits 0..1), after which each step is a byte move,
// one logic op for the slot offset, the load and the XOR.
__device__ __forceinline__ gf128 gf_mul_tab(const uint4* __restrict__ T, const gf128& y, uint32_t rot) {
  rot &= 7;
  // permuted byte st of yp = byte st ^ rot of y
  const bool sw = rot & 4;
  uint32_t yp[4] = {sw ? y.w[1] : y.w[0], sw ? y.w[0] : y.w[1], sw ? y.w[3] : y.w[2], sw ? y.w[2] : y.w[3]};
  const uint32_t x3 = rot & 3;
  const uint32_t perm = x3 == 0 ? 0x3210u : x3 == 1 ? 0x2301u : x3 == 2 ? 0x1032u : 0x0123u;
#pragma unroll
  for (int i = 0; i < 4; i++) yp[i] = __byte_perm(yp[i], 0, perm);
  const uint32_t xk = rot << 4;  // byte offset of the position XOR
  const char* base = reinterpret_cast<const char*>(T);
  uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll
  for (int st = 0; st < 16; st++) {
    // byte st of yp placed at bits 8..15 = v << 8; slot (v << 4) | (st ^ rot) is
    // byte offset (v << 8) | ((st ^ rot) << 4)
    const uint32_t vb = __byte_perm(yp[st >> 2], 0, 0x4404u | ((uint32_t)(st & 3) << 4));
    const uint32_t off = (vb | ((uint32_t)st << 4)) ^ xk;
    const uint4 v = *reinterpret_cast<const uint4*>(base + off);
    a0 ^= v.x; a1 ^= v.y; a2 ^= v.z; a3 ^= v.w;
  }
  gf128 o;
  o.w[0] = a0; o.w[1] = a1; o.w[2] = a2; o.w[3] = a3;
  return o;
}

__host__ __device__ constexpr int gf_tab_ctz4(int j) { return (j & 1) ? 0 : (j & 2) ? 1 : (j & 4) ? 2 : 3; }

// One row of the byte table computed directly, without nibble tables or a
// barrier: item = g << 4 | k (g, k < 16) writes the 16 slots (v << 4) + k of
// v = 16 g + j, j < 16, i.e. t v x^(8k) = L_k(j) + H_k(g) with L_k(j) the sum
// of t x^(8k+b) over the bits b of j and H_k(g) that of t x^(8k+4+b) over the
// bits of g. The eight images t x^(8k+b) come from one shift and seven
// doublings; j walks the Gray code, one XOR per slot. Every thread works from
// the start (measured faster than building 16-entry nibble tables first, whose
// serial phase leaves most warps waiting, and with 16 B fewer shared-memory
// reads per slot). Eight consecutive items have eight consecutive k, so their
// writes hit distinct bank groups.
__device__ __forceinline__ void gf_tab_row_direct(gf128 t, uint4* __restrict__ T, int item) {
  const int g = (item >> 4) & 15, k = item & 15;
  gf128 B[8];
  B[0] = gf_mul_xpow_small(t, 8 * k);
#pragma unroll
  for (int b = 1; b < 8; b++) B[b] = gf_mul_x(B[b - 1]);
  gf128 v = gf_zero();
#pragma unroll
  for (int b = 0; b < 4; b++) {
    const uint32_t m = 0u - (uint32_t)((g >> b) & 1);
#pragma unroll
    for (int w = 0; w < 4; w++) v.w[w] ^= B[4 + b].w[w] & m;
  }
  uint4* row = T + (g << 8) + k;
#pragma unroll
  for (int jj = 0; jj < 16; jj++) {
    if (jj) v = gf_add(v, B[gf_tab_ctz4(jj)]);
    const int j = jj ^ (jj >> 1);
    row[j << 4] = make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]);
  }
}

// Byte tables of one multiplier t into T (GF_TAB_ENTRIES slots): all threads
// of the CTA call it (any block size); it ends with a barrier, after which T
// is ready.
__device__ __forceinline__ void gf_tab_build(gf128 t, uint4* __restrict__ T) {
  for (int it = threadIdx.x; it < 256; it += blockDim.x) gf_tab_row_direct(t, T, it);
  __syncthreads();
}

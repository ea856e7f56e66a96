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
constexpr int GF_TAB_NIBBLE_SLOTS = 2 * 256;  // slots of its nibble tables

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

// Nibble tables of t into LH (GF_TAB_NIBBLE_SLOTS slots): L[j][k] = t j x^(8k)
// at j * 16 + k and H[g][k] = t g x^(8k + 4) at 256 + g * 16 + k, for nibbles
// j, g < 16. Called by 32 threads, part = 0..31 (k = part & 15, L or H by
// part >> 4), each with a Gray-code walk over four images t x^i.
__device__ __forceinline__ void gf_tab_nibbles(gf128 t, uint4* __restrict__ LH, int part) {
  const int half = part >> 4, k = part & 15;
  gf128 B[4];
#pragma unroll
  for (int b = 0; b < 4; b++) B[b] = gf_mul_xpow_small(t, 8 * k + 4 * half + b);
  gf128 v[16];
  v[0] = gf_zero();
#pragma unroll
  for (int j = 1; j < 16; j++) v[j] = gf_add(v[j & (j - 1)], B[gf_tab_ctz4(j)]);
  uint4* out = LH + half * 256;
#pragma unroll
  for (int j = 0; j < 16; j++) out[j * 16 + k] = make_uint4(v[j].w[0], v[j].w[1], v[j].w[2], v[j].w[3]);
}

// Part of the byte table from the nibble tables, by rows: item = s * 256 +
// (g << 4 | k) writes the 16 / SPLIT slots (v << 4) + k of v = 16 g + j, j in
// part s of 0..15, as L[j][k] + H[g][k] with H[g][k] read once (a third fewer
// shared-memory accesses than entry by entry). Eight consecutive items have
// eight consecutive k, so their reads and writes hit distinct bank groups.
template <int SPLIT>
__device__ __forceinline__ void gf_tab_rows(const uint4* __restrict__ LH, uint4* __restrict__ T, int item) {
  constexpr int J = 16 / SPLIT;
  const int s = item >> 8, g = (item >> 4) & 15, k = item & 15;
  const uint4 h = LH[256 + g * 16 + k];
#pragma unroll
  for (int jj = 0; jj < J; jj++) {
    const int j = s * J + jj;
    const uint4 l = LH[j * 16 + k];
    T[((16 * g + j) << 4) + k] = make_uint4(l.x ^ h.x, l.y ^ h.y, l.z ^ h.z, l.w ^ h.w);
  }
}

// One row of the byte table computed directly, without nibble tables or a
// barrier: item = g << 4 | k (g, k < 16) writes the 16 slots (v << 4) + k of
// v = 16 g + j, j < 16, i.e. t v x^(8k) = L_k(j) + H_k(g) with L_k(j) the sum
// of t x^(8k+b) over the bits b of j and H_k(g) that of t x^(8k+4+b) over the
// bits of g. The eight images t x^(8k+b) come from one shift and seven
// doublings; j walks the Gray code, one XOR per slot. Suits tables rebuilt
// often (one multiplier after another): every thread works, nothing waits on
// a serial nibble phase. Eight consecutive items have eight consecutive k,
// so their writes hit distinct bank groups.
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

// Byte tables of one multiplier t into T (GF_TAB_ENTRIES slots), using LH
// (GF_TAB_NIBBLE_SLOTS slots) as scratch. All threads of the CTA call it; it
// ends with a barrier, after which T is ready.
__device__ __forceinline__ void gf_tab_build(gf128 t, uint4* __restrict__ T, uint4* __restrict__ LH) {
  if (threadIdx.x < 32) gf_tab_nibbles(t, LH, threadIdx.x);
  __syncthreads();
  for (int it = threadIdx.x; it < 256; it += blockDim.x) gf_tab_rows<1>(LH, T, it);
  __syncthreads();
}

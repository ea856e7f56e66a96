// GF(2^128) arithmetic on the device.
//
// Field: polynomial basis modulo x^128 + x^7 + x^2 + x + 1 (the reference's
// GHASH form, crates/flock-core/src/field/gf2_128.rs:1-135). An element is
// four little-endian 32-bit limbs, limb 0 holding x^0..x^31.
//
// The GPU has no carry-less multiply instruction. A 32x32 carry-less product
// is formed from sixteen 32x32->64 integer multiplies of operands masked to
// every fourth bit: with four-bit spacing each output position sums at most
// eight partial bits, so the count never carries into the next position of
// the same residue class, and keeping the residue's bits keeps the parity.
// 128x128 uses two levels of Karatsuba (nine 32-bit products) and the
// reference's fold of the upper half (gf2_128.rs:192-216).
#pragma once
#include <cstdint>

struct __align__(16) gf128 {
  uint32_t w[4];
};

__host__ __device__ __forceinline__ gf128 gf_zero() { gf128 r; r.w[0] = r.w[1] = r.w[2] = r.w[3] = 0; return r; }
__host__ __device__ __forceinline__ gf128 gf_one() { gf128 r = gf_zero(); r.w[0] = 1; return r; }
__host__ __device__ __forceinline__ gf128 gf_add(gf128 a, gf128 b) {
  gf128 r;
  r.w[0] = a.w[0] ^ b.w[0]; r.w[1] = a.w[1] ^ b.w[1]; r.w[2] = a.w[2] ^ b.w[2]; r.w[3] = a.w[3] ^ b.w[3];
  return r;
}
__host__ __device__ __forceinline__ bool gf_eq(gf128 a, gf128 b) {
  return ((a.w[0] ^ b.w[0]) | (a.w[1] ^ b.w[1]) | (a.w[2] ^ b.w[2]) | (a.w[3] ^ b.w[3])) == 0;
}

__device__ __forceinline__ gf128 gf_load(const void* p) {
  uint4 v = *reinterpret_cast<const uint4*>(p);
  gf128 r; r.w[0] = v.x; r.w[1] = v.y; r.w[2] = v.z; r.w[3] = v.w;
  return r;
}
__device__ __forceinline__ void gf_store(void* p, gf128 a) {
  *reinterpret_cast<uint4*>(p) = make_uint4(a.w[0], a.w[1], a.w[2], a.w[3]);
}

// 32x32 -> 64 unsigned integer product (one IMAD.WIDE.U32).
__device__ __forceinline__ uint64_t mulw(uint32_t a, uint32_t b) {
  uint64_t r;
  asm("mul.wide.u32 %0, %1, %2;" : "=l"(r) : "r"(a), "r"(b));
  return r;
}

// 32x32 -> 64 unsigned multiply-add (one IMAD.WIDE.U32 with accumulator).
__device__ __forceinline__ uint64_t madw(uint32_t a, uint32_t b, uint64_t c) {
  uint64_t r;
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"(a), "r"(b), "l"(c));
  return r;
}

// (x & ~m) | (y & m): one 3-input logic op.
__device__ __forceinline__ uint32_t bit_select(uint32_t x, uint32_t y, uint32_t m) { return (x & ~m) | (y & m); }

// Combines the four residue-class partial products: class k keeps the bits at
// positions = k (mod 4). Selecting per class (instead of masking each and
// OR-ing) is three logic ops per 32-bit half.
__device__ __forceinline__ uint64_t clmul_combine(uint64_t r0, uint64_t r1, uint64_t r2, uint64_t r3) {
  const uint32_t m1 = 0x22222222u, m3 = 0x88888888u, m23 = 0xCCCCCCCCu;
  const uint32_t lo = bit_select(bit_select((uint32_t)r0, (uint32_t)r1, m1), bit_select((uint32_t)r2, (uint32_t)r3, m3), m23);
  const uint32_t hi = bit_select(bit_select((uint32_t)(r0 >> 32), (uint32_t)(r1 >> 32), m1),
                                 bit_select((uint32_t)(r2 >> 32), (uint32_t)(r3 >> 32), m3), m23);
  return ((uint64_t)hi << 32) | lo;
}

// 32x32 -> 64 carry-less product of a and the four masked parts (b0..b3) of b.
// Products of operands masked to every fourth bit hold, at each position, the
// count of its partial bits (at most 8), so the count's low bit is the XOR.
// Two products whose counts sit in neighbouring columns of the same residue
// class (offsets i + j and i + j + 4) sum to at most 15 per column, so such
// pairs are added by the multiplier's accumulator instead of an XOR.
__device__ __forceinline__ uint64_t clmul32_m(uint32_t a, uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3) {
  const uint32_t m0 = 0x11111111u, m1 = 0x22222222u, m2 = 0x44444444u, m3 = 0x88888888u;
  const uint32_t a0 = a & m0, a1 = a & m1, a2 = a & m2, a3 = a & m3;
  const uint64_t r0 = madw(a0, b0, mulw(a1, b3)) ^ mulw(a2, b2) ^ mulw(a3, b1);
  const uint64_t r1 = madw(a0, b1, mulw(a2, b3)) ^ madw(a1, b0, mulw(a3, b2));
  const uint64_t r2 = madw(a0, b2, mulw(a3, b3)) ^ mulw(a1, b1) ^ mulw(a2, b0);
  const uint64_t r3 = mulw(a0, b3) ^ mulw(a1, b2) ^ mulw(a2, b1) ^ mulw(a3, b0);
  return clmul_combine(r0, r1, r2, r3);
}

// 32x32 -> 64 carry-less product.
__device__ __forceinline__ uint64_t clmul32(uint32_t a, uint32_t b) {
  return clmul32_m(a, b & 0x11111111u, b & 0x22222222u, b & 0x44444444u, b & 0x88888888u);
}

// 64x64 -> 128 carry-less product (Karatsuba over 32-bit halves).
__device__ __forceinline__ void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  uint32_t al = (uint32_t)a, ah = (uint32_t)(a >> 32), bl = (uint32_t)b, bh = (uint32_t)(b >> 32);
  uint64_t ll = clmul32(al, bl), hh = clmul32(ah, bh), mm = clmul32(al ^ ah, bl ^ bh);
  mm ^= ll ^ hh;
  lo = ll ^ (mm << 32);
  hi = hh ^ (mm >> 32);
}

// Fold bits 128..255 back: x^128 = x^7 + x^2 + x + 1.
__device__ __forceinline__ gf128 gf_reduce(uint64_t r0, uint64_t r1, uint64_t r2, uint64_t r3) {
  uint64_t t_lo = r2 ^ (r2 << 1) ^ (r2 << 2) ^ (r2 << 7);
  uint64_t t_hi = r3 ^ ((r3 << 1) | (r2 >> 63)) ^ ((r3 << 2) | (r2 >> 62)) ^ ((r3 << 7) | (r2 >> 57));
  uint64_t ov = (r3 >> 63) ^ (r3 >> 62) ^ (r3 >> 57);
  uint64_t corr = ov ^ (ov << 1) ^ (ov << 2) ^ (ov << 7);
  uint64_t lo = r0 ^ t_lo ^ corr, hi = r1 ^ t_hi;
  gf128 r;
  r.w[0] = (uint32_t)lo; r.w[1] = (uint32_t)(lo >> 32); r.w[2] = (uint32_t)hi; r.w[3] = (uint32_t)(hi >> 32);
  return r;
}

// Unreduced 256-bit product (Karatsuba over 64-bit halves).
struct gf256 {
  uint64_t r[4];
};
__device__ __forceinline__ gf256 gf_mul_wide(gf128 a, gf128 b) {
  uint64_t alo = a.w[0] | ((uint64_t)a.w[1] << 32), ahi = a.w[2] | ((uint64_t)a.w[3] << 32);
  uint64_t blo = b.w[0] | ((uint64_t)b.w[1] << 32), bhi = b.w[2] | ((uint64_t)b.w[3] << 32);
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul64(alo, blo, l0, l1);
  clmul64(ahi, bhi, h0, h1);
  clmul64(alo ^ ahi, blo ^ bhi, m0, m1);
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  gf256 o;
  o.r[0] = l0;
  o.r[1] = l1 ^ m0;
  o.r[2] = h0 ^ m1;
  o.r[3] = h1;
  return o;
}
__device__ __forceinline__ void gf256_acc(gf256& acc, const gf256& x) {
  acc.r[0] ^= x.r[0]; acc.r[1] ^= x.r[1]; acc.r[2] ^= x.r[2]; acc.r[3] ^= x.r[3];
}
__device__ __forceinline__ gf128 gf256_reduce(const gf256& x) { return gf_reduce(x.r[0], x.r[1], x.r[2], x.r[3]); }

__device__ __forceinline__ gf128 gf_mul(gf128 a, gf128 b) { return gf256_reduce(gf_mul_wide(a, b)); }

// Multiply by x.
__device__ __forceinline__ gf128 gf_mul_x(gf128 a) {
  uint32_t carry = a.w[3] >> 31;
  gf128 r;
  r.w[3] = (a.w[3] << 1) | (a.w[2] >> 31);
  r.w[2] = (a.w[2] << 1) | (a.w[1] >> 31);
  r.w[1] = (a.w[1] << 1) | (a.w[0] >> 31);
  r.w[0] = (a.w[0] << 1) ^ (0x87u & (0u - carry));
  return r;
}

// ---- products by a prepared operand ------------------------------------------
// When one factor is reused (an NTT twiddle, an eq weight), its nine Karatsuba
// words (b0, b1, b0^b1, b2, b3, b2^b3, b0^b2, b1^b3, b0^b1^b2^b3), each split
// into the four every-fourth-bit masks, can be computed once and stored: a
// product with the prepared form skips that masking (36 logic instructions).
struct __align__(16) gf128p {
  uint4 m[9];
};

__host__ __device__ inline gf128p gf_prepare(gf128 b) {
  const uint32_t w[9] = {b.w[0], b.w[1], b.w[0] ^ b.w[1], b.w[2], b.w[3], b.w[2] ^ b.w[3],
                         b.w[0] ^ b.w[2], b.w[1] ^ b.w[3], b.w[0] ^ b.w[1] ^ b.w[2] ^ b.w[3]};
  gf128p p;
  for (int i = 0; i < 9; i++)
    p.m[i] = make_uint4(w[i] & 0x11111111u, w[i] & 0x22222222u, w[i] & 0x44444444u, w[i] & 0x88888888u);
  return p;
}

__device__ __forceinline__ uint64_t clmul32_p(uint32_t a, uint4 b) { return clmul32_m(a, b.x, b.y, b.z, b.w); }

__device__ __forceinline__ gf256 gf_mul_wide_p(gf128 a, const gf128p& p) {
  const uint32_t a0 = a.w[0], a1 = a.w[1], a2 = a.w[2], a3 = a.w[3];
  uint64_t ll = clmul32_p(a0, p.m[0]), lh = clmul32_p(a1, p.m[1]), lm = clmul32_p(a0 ^ a1, p.m[2]);
  lm ^= ll ^ lh;
  const uint64_t l0 = ll ^ (lm << 32), l1 = lh ^ (lm >> 32);
  uint64_t hl = clmul32_p(a2, p.m[3]), hh = clmul32_p(a3, p.m[4]), hm = clmul32_p(a2 ^ a3, p.m[5]);
  hm ^= hl ^ hh;
  const uint64_t h0 = hl ^ (hm << 32), h1 = hh ^ (hm >> 32);
  const uint32_t c0 = a0 ^ a2, c1 = a1 ^ a3;
  uint64_t ml = clmul32_p(c0, p.m[6]), mh = clmul32_p(c1, p.m[7]), mx = clmul32_p(c0 ^ c1, p.m[8]);
  mx ^= ml ^ mh;
  uint64_t m0 = ml ^ (mx << 32), m1 = mh ^ (mx >> 32);
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  gf256 o;
  o.r[0] = l0; o.r[1] = l1 ^ m0; o.r[2] = h0 ^ m1; o.r[3] = h1;
  return o;
}
__device__ __forceinline__ gf128 gf_mul_p(gf128 a, const gf128p& p) { return gf256_reduce(gf_mul_wide_p(a, p)); }

// a * b for a multiplier below 2^32, from the masks of its low word (m[0] of
// its prepared form): four 32-bit products, a 160-bit result.
__device__ __forceinline__ gf128 gf_mul_p32(gf128 a, uint4 m0) {
  const uint64_t p0 = clmul32_p(a.w[0], m0), p1 = clmul32_p(a.w[1], m0);
  const uint64_t p2 = clmul32_p(a.w[2], m0), p3 = clmul32_p(a.w[3], m0);
  return gf_reduce(p0 ^ (p1 << 32), (p1 >> 32) ^ p2 ^ (p3 << 32), p3 >> 32, 0);
}

// a * b for a multiplier below 2^64, from m[0..2] of its prepared form (the
// masks of b0, b1, b0 ^ b1): a's two 64-bit halves times b by Karatsuba over
// 32-bit words, six 32-bit products, a 192-bit result.
__device__ __forceinline__ gf128 gf_mul_p64(gf128 a, uint4 m0, uint4 m1, uint4 m2) {
  const uint64_t ll = clmul32_p(a.w[0], m0), lh = clmul32_p(a.w[1], m1);
  const uint64_t lm = clmul32_p(a.w[0] ^ a.w[1], m2) ^ ll ^ lh;
  const uint64_t hl = clmul32_p(a.w[2], m0), hh = clmul32_p(a.w[3], m1);
  const uint64_t hm = clmul32_p(a.w[2] ^ a.w[3], m2) ^ hl ^ hh;
  const uint64_t l0 = ll ^ (lm << 32), l1 = lh ^ (lm >> 32), h0 = hl ^ (hm << 32), h1 = hh ^ (hm >> 32);
  return gf_reduce(l0, l1 ^ h0, h1, 0);
}
// a * t for t below 2^40 given the prepared low 32 bits of t (m0, as
// gf_mul_p32) and its bits 32..39 (thi): the four 32-bit products plus one
// copy of a shifted by 32 + j per set bit j of thi (the same in every lane of
// a layer's block, so the loop does not diverge).
__device__ __forceinline__ gf128 gf_mul_p40(gf128 a, uint4 m0, uint32_t thi) {
  const uint64_t p0 = clmul32_p(a.w[0], m0), p1 = clmul32_p(a.w[1], m0);
  const uint64_t p2 = clmul32_p(a.w[2], m0), p3 = clmul32_p(a.w[3], m0);
  uint64_t r0 = p0 ^ (p1 << 32), r1 = (p1 >> 32) ^ p2 ^ (p3 << 32), r2 = p3 >> 32;
  const uint64_t alo = a.w[0] | ((uint64_t)a.w[1] << 32), ahi = a.w[2] | ((uint64_t)a.w[3] << 32);
  for (uint32_t t = thi; t; t &= t - 1) {
    const int s = 32 + __ffs(t) - 1;  // 32 <= s < 40
    r0 ^= alo << s;
    r1 ^= (ahi << s) | (alo >> (64 - s));
    r2 ^= ahi >> (64 - s);
  }
  return gf_reduce(r0, r1, r2, 0);
}

// a * t for t below 2^72 given the prepared low 64 bits of t (m0, m1, m2, as
// gf_mul_p64) and its bits 64..71 (thi): the 64-bit product's 192 bits plus
// a * thi placed at bit 64, one shifted copy of a per set bit of thi (thi is
// the same in every lane of a layer's block, so the loop does not diverge).
__device__ __forceinline__ gf128 gf_mul_p72(gf128 a, uint4 m0, uint4 m1, uint4 m2, uint32_t thi) {
  const uint64_t ll = clmul32_p(a.w[0], m0), lh = clmul32_p(a.w[1], m1);
  const uint64_t lm = clmul32_p(a.w[0] ^ a.w[1], m2) ^ ll ^ lh;
  const uint64_t hl = clmul32_p(a.w[2], m0), hh = clmul32_p(a.w[3], m1);
  const uint64_t hm = clmul32_p(a.w[2] ^ a.w[3], m2) ^ hl ^ hh;
  uint64_t r1 = lh ^ (lm >> 32) ^ hl ^ (hm << 32), r2 = hh ^ (hm >> 32), r3 = 0;
  const uint64_t alo = a.w[0] | ((uint64_t)a.w[1] << 32), ahi = a.w[2] | ((uint64_t)a.w[3] << 32);
  for (uint32_t t = thi; t; t &= t - 1) {
    const int j = __ffs(t) - 1;
    r1 ^= alo << j;
    r2 ^= (ahi << j) | (j ? alo >> (64 - j) : 0);
    r3 ^= j ? ahi >> (64 - j) : 0;
  }
  return gf_reduce(ll ^ (lm << 32), r1, r2, r3);
}
__device__ __forceinline__ gf128p gf_load_p(const gf128p* q) {
  gf128p p;
#pragma unroll
  for (int i = 0; i < 9; i++) p.m[i] = q->m[i];
  return p;
}

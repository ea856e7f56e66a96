// Host-side GF(2^128) / GF(2^8) arithmetic for setup-time tables and the
// Fiat-Shamir side of the prover (transcript values, small sumcheck tails).
// Same field as the device code: polynomial basis mod x^128 + x^7 + x^2 + x + 1
// (crates/flock-core/src/field/gf2_128.rs:1-135).
#pragma once
#include <cstdint>
#include <vector>

#if defined(__aarch64__) && (defined(__ARM_FEATURE_AES) || defined(__ARM_FEATURE_CRYPTO))
#define FLOCK_HOST_PMULL 1
// 64x64 carry-less product by the Arm PMULL instruction (host_pmull.cpp).
void flock_host_clmul64(uint64_t a, uint64_t b, uint64_t* lo, uint64_t* hi);
#else
#define FLOCK_HOST_PMULL 0
#endif

namespace hf {

struct F {
  uint64_t lo = 0, hi = 0;
  F() = default;
  constexpr F(uint64_t l, uint64_t h) : lo(l), hi(h) {}
  static F one() { return F(1, 0); }
  bool operator==(const F& o) const { return lo == o.lo && hi == o.hi; }
  bool operator!=(const F& o) const { return !(*this == o); }
  F operator+(const F& o) const { return F(lo ^ o.lo, hi ^ o.hi); }
  F& operator+=(const F& o) { lo ^= o.lo; hi ^= o.hi; return *this; }
  bool zero() const { return (lo | hi) == 0; }
};

// 32x32 -> 64 carry-less product by integer multiplies of operands masked to
// every fourth bit: a column of a masked product counts at most 8 partial
// bits, so the count never reaches the next column of its residue class and
// the column's low bit is their XOR (the same device trick as in gf128.cuh;
// portable C++, 10x the 4-bit window method it replaced).
inline uint64_t clmul32(uint32_t a, uint32_t b) {
  const uint32_t m0 = 0x11111111u, m1 = 0x22222222u, m2 = 0x44444444u, m3 = 0x88888888u;
  const uint64_t a0 = a & m0, a1 = a & m1, a2 = a & m2, a3 = a & m3;
  const uint64_t b0 = b & m0, b1 = b & m1, b2 = b & m2, b3 = b & m3;
  const uint64_t r0 = (a0 * b0) ^ (a1 * b3) ^ (a2 * b2) ^ (a3 * b1);
  const uint64_t r1 = (a0 * b1) ^ (a1 * b0) ^ (a2 * b3) ^ (a3 * b2);
  const uint64_t r2 = (a0 * b2) ^ (a1 * b1) ^ (a2 * b0) ^ (a3 * b3);
  const uint64_t r3 = (a0 * b3) ^ (a1 * b2) ^ (a2 * b1) ^ (a3 * b0);
  const uint64_t M0 = 0x1111111111111111ull, M1 = M0 << 1, M2 = M0 << 2, M3 = M0 << 3;
  return (r0 & M0) | (r1 & M1) | (r2 & M2) | (r3 & M3);
}

#if FLOCK_HOST_PMULL
// An Arm host built with the crypto extension multiplies with PMULL: the same
// value as the portable form below, several times faster on a Grace core.
inline void clmul(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) { flock_host_clmul64(a, b, &lo, &hi); }
#else
// 64x64 carry-less product (Karatsuba over 32-bit halves).
inline void clmul(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  const uint32_t al = (uint32_t)a, ah = (uint32_t)(a >> 32), bl = (uint32_t)b, bh = (uint32_t)(b >> 32);
  const uint64_t ll = clmul32(al, bl), hh = clmul32(ah, bh);
  const uint64_t mm = clmul32(al ^ ah, bl ^ bh) ^ ll ^ hh;
  lo = ll ^ (mm << 32);
  hi = hh ^ (mm >> 32);
}
#endif

inline F reduce(uint64_t r0, uint64_t r1, uint64_t r2, uint64_t r3) {
  uint64_t t_lo = r2 ^ (r2 << 1) ^ (r2 << 2) ^ (r2 << 7);
  uint64_t t_hi = r3 ^ ((r3 << 1) | (r2 >> 63)) ^ ((r3 << 2) | (r2 >> 62)) ^ ((r3 << 7) | (r2 >> 57));
  uint64_t ov = (r3 >> 63) ^ (r3 >> 62) ^ (r3 >> 57);
  uint64_t corr = ov ^ (ov << 1) ^ (ov << 2) ^ (ov << 7);
  return F(r0 ^ t_lo ^ corr, r1 ^ t_hi);
}

inline F operator*(F a, F b) {
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul(a.lo, b.lo, l0, l1);
  clmul(a.hi, b.hi, h0, h1);
  clmul(a.lo ^ a.hi, b.lo ^ b.hi, m0, m1);
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  return reduce(l0, l1 ^ m0, h0 ^ m1, h1);
}
inline F& operator*=(F& a, F b) { a = a * b; return a; }

inline F inv(F a) {
  F r = F::one(), cur = a * a;
  for (int i = 1; i < 128; i++) { r = r * cur; cur = cur * cur; }
  return r;
}

// GF(2^8) with modulus x^8 + x^4 + x^3 + x + 1 and its embedding into
// GF(2^128). The embedding is the field homomorphism sending the GF(2^8)
// element 0x02 to the GF(2^128) value of crates/flock-core/src/field/phi8.rs:29-30.
inline uint8_t f8_mul(uint8_t a, uint8_t b) {
  unsigned acc = 0;
  for (int i = 0; i < 8; i++)
    if ((a >> i) & 1) acc ^= (unsigned)b << i;
  for (int i = 14; i >= 8; i--)
    if ((acc >> i) & 1) acc ^= 0x11Bu << (i - 8);
  return (uint8_t)acc;
}
inline const F* phi8_table() {
  static const std::vector<F> t = [] {
    std::vector<F> v(256);
    F g(0x6b8330483c2e9849ULL, 0x0dcb364640a222feULL), p[8];
    p[0] = F::one();
    for (int i = 1; i < 8; i++) p[i] = p[i - 1] * g;
    for (int x = 0; x < 256; x++) {
      F acc;
      for (int i = 0; i < 8; i++)
        if ((x >> i) & 1) acc += p[i];
      v[x] = acc;
    }
    return v;
  }();
  return t.data();
}
inline F phi8(uint8_t v) { return phi8_table()[v]; }

}  // namespace hf

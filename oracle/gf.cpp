// GF(2^128) / GF(2^8) arithmetic for the oracle (test infrastructure only).
#include "oracle.h"

#if defined(__aarch64__) && (defined(__ARM_FEATURE_AES) || defined(__ARM_FEATURE_CRYPTO))
#include <arm_neon.h>
#endif

namespace oracle {

// 64x64 -> 128 carry-less products. Same value as the reference's bit-serial
// clmul64 (crates/flock-core/src/field/gf2_128/portable.rs:4-20).
//
// Portable form: a 4-bit window table of b.
static inline void clmul64_portable(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  uint64_t tl[16], th[16];
  tl[0] = 0; th[0] = 0;
  tl[1] = b; th[1] = 0;
  tl[2] = b << 1; th[2] = b >> 63;
  tl[4] = b << 2; th[4] = b >> 62;
  tl[8] = b << 3; th[8] = b >> 61;
  for (int n = 3; n < 16; n++) {
    if ((n & (n - 1)) == 0) continue;
    int low = n & -n;
    tl[n] = tl[low] ^ tl[n ^ low];
    th[n] = th[low] ^ th[n ^ low];
  }
  lo = 0; hi = 0;
  for (int i = 15; i >= 0; i--) {
    hi = (hi << 4) | (lo >> 60);
    lo <<= 4;
    unsigned nib = (unsigned)(a >> (4 * i)) & 15u;
    lo ^= tl[nib];
    hi ^= th[nib];
  }
}

#if defined(__aarch64__) && (defined(__ARM_FEATURE_AES) || defined(__ARM_FEATURE_CRYPTO))
// The reference's aarch64 backend multiplies with PMULL
// (crates/flock-core/src/field/gf2_128/aarch64.rs:26-60); so does the oracle
// on an Arm host built with the crypto extension (oracle/Makefile).
#define ORACLE_GF_PMULL 1
static inline void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  const poly128_t p = vmull_p64((poly64_t)a, (poly64_t)b);
  const uint64x2_t v = vreinterpretq_u64_p128(p);
  lo = vgetq_lane_u64(v, 0);
  hi = vgetq_lane_u64(v, 1);
}
#else
#define ORACLE_GF_PMULL 0
static inline void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) { clmul64_portable(a, b, lo, hi); }
#endif

// crates/flock-core/src/field/gf2_128.rs:192-216 (fold of the upper 128 bits).
static inline F128 reduce(uint64_t r0, uint64_t r1, uint64_t r2, uint64_t r3) {
  uint64_t s1_lo = r2 << 1, s1_hi = (r3 << 1) | (r2 >> 63);
  uint64_t s2_lo = r2 << 2, s2_hi = (r3 << 2) | (r2 >> 62);
  uint64_t s7_lo = r2 << 7, s7_hi = (r3 << 7) | (r2 >> 57);
  uint64_t t_lo = r2 ^ s1_lo ^ s2_lo ^ s7_lo;
  uint64_t t_hi = r3 ^ s1_hi ^ s2_hi ^ s7_hi;
  uint64_t ov = (r3 >> 63) ^ (r3 >> 62) ^ (r3 >> 57);
  uint64_t corr = ov ^ (ov << 1) ^ (ov << 2) ^ (ov << 7);
  return f128(r0 ^ t_lo ^ corr, r1 ^ t_hi);
}

F128 gf_mul(F128 a, F128 b) {
  uint64_t ll_lo, ll_hi, lh_lo, lh_hi, hl_lo, hl_hi, hh_lo, hh_hi;
  clmul64(a.lo, b.lo, ll_lo, ll_hi);
  clmul64(a.lo, b.hi, lh_lo, lh_hi);
  clmul64(a.hi, b.lo, hl_lo, hl_hi);
  clmul64(a.hi, b.hi, hh_lo, hh_hi);
  uint64_t cr_lo = lh_lo ^ hl_lo, cr_hi = lh_hi ^ hl_hi;
  return reduce(ll_lo, ll_hi ^ cr_lo, hh_lo ^ cr_hi, hh_hi);
}

// The portable product whatever the host; the test suite checks it against
// gf_mul (PMULL on an Arm host with the crypto extension).
F128 gf_mul_portable(F128 a, F128 b) {
  uint64_t ll_lo, ll_hi, lh_lo, lh_hi, hl_lo, hl_hi, hh_lo, hh_hi;
  clmul64_portable(a.lo, b.lo, ll_lo, ll_hi);
  clmul64_portable(a.lo, b.hi, lh_lo, lh_hi);
  clmul64_portable(a.hi, b.lo, hl_lo, hl_hi);
  clmul64_portable(a.hi, b.hi, hh_lo, hh_hi);
  uint64_t cr_lo = lh_lo ^ hl_lo, cr_hi = lh_hi ^ hl_hi;
  return reduce(ll_lo, ll_hi ^ cr_lo, hh_lo ^ cr_hi, hh_hi);
}

int gf_mul_uses_pmull() { return ORACLE_GF_PMULL; }

// Fermat inverse a^(2^128-2), gf2_128.rs:56-66.
F128 gf_inv(F128 a) {
  F128 r = f128(1);
  F128 cur = a * a;
  for (int i = 1; i < 128; i++) {
    r = r * cur;
    cur = cur * cur;
  }
  return r;
}

// gf2_128.rs:117-125
F128 gf_mul_x(F128 z) {
  uint64_t carry = z.hi >> 63;
  uint64_t mask = 0 - carry;
  return f128((z.lo << 1) ^ (0x87 & mask), (z.hi << 1) | (z.lo >> 63));
}

uint8_t gf8_mul(uint8_t a, uint8_t b) {
  uint16_t acc = 0;
  for (int i = 0; i < 8; i++)
    if ((a >> i) & 1) acc ^= (uint16_t)(b << i);
  for (int i = 14; i >= 8; i--)
    if ((acc >> i) & 1) acc ^= (uint16_t)(0x11B << (i - 8));
  return (uint8_t)acc;
}

uint8_t gf8_inv(uint8_t a) {
  uint8_t r = 1, sq = a;
  for (int i = 0; i < 8; i++) {
    if ((0xFE >> i) & 1) r = gf8_mul(r, sq);
    sq = gf8_mul(sq, sq);
  }
  return r;
}

// phi8 is the field homomorphism GF(2^8) -> GF(2^128) fixed by the image of
// the GF(2^8) element x (0x02). That image is entry 2 of PHI_8_TABLE at
// crates/flock-core/src/field/phi8.rs:29-30; the other 255 entries follow by
// linearity: phi8(v) = sum_i bit_i(v) * g^i.
static const F128* phi8_table() {
  static const std::vector<F128> table = [] {
    std::vector<F128> t(256);
    F128 g = f128(0x6b8330483c2e9849ULL, 0x0dcb364640a222feULL);
    F128 pw[8];
    pw[0] = f128(1);
    for (int i = 1; i < 8; i++) pw[i] = pw[i - 1] * g;
    for (int x = 0; x < 256; x++) {
      F128 acc;
      for (int i = 0; i < 8; i++)
        if ((x >> i) & 1) acc += pw[i];
      t[x] = acc;
    }
    return t;
  }();
  return table.data();
}

F128 phi8(uint8_t v) { return phi8_table()[v]; }

}  // namespace oracle

// Constant tables of the zerocheck round-1 kernel, built once on the host.
#pragma once
#include <cstdint>
#include <vector>

#include "host_field.h"

struct ZcRound1Tables {
  // ext[c][v][j]: bit i = bit j of ext_i(v << 8c), the GF(2^8) value at
  // lambda_i = 64 + i of the degree<64 interpolant of the bits v placed at
  // skip positions 8c..8c+7 (zerocheck/univariate_skip.rs:84-138).
  uint64_t ext[8][256][8];
  uint64_t phi8[256][2];  // phi8 embedding GF(2^8) -> GF(2^128), [lo, hi]
  uint8_t e8[8];          // GF(2^8) eq weight of the three fixed small challenges
  uint8_t e8c[4];         // GF(2^8) eq weight of the fixed challenges r7, r8 (c statistic)
};

namespace zc {

// Fixed inner challenges (zerocheck/univariate_skip_optimized.rs:85-120).
constexpr uint8_t SMALL_CHAL[3] = {0xF7, 0x53, 0xB5};

// M[i][s] = L_s(64 + i) over GF(2^8) with nodes S = {0..63}.
inline std::vector<uint8_t> ext_matrix() {
  std::vector<uint8_t> M(64 * 64);
  auto inv = [](uint8_t a) {
    uint8_t r = 1, sq = a;
    for (int i = 0; i < 8; i++) {
      if ((0xFE >> i) & 1) r = hf::f8_mul(r, sq);
      sq = hf::f8_mul(sq, sq);
    }
    return r;
  };
  for (int i = 0; i < 64; i++)
    for (int s = 0; s < 64; s++) {
      uint8_t num = 1, den = 1, lam = (uint8_t)(64 + i);
      for (int t = 0; t < 64; t++) {
        if (t == s) continue;
        num = hf::f8_mul(num, lam ^ (uint8_t)t);
        den = hf::f8_mul(den, (uint8_t)(s ^ t));
      }
      M[i * 64 + s] = hf::f8_mul(num, inv(den));
    }
  return M;
}

inline uint8_t e8(int xs) {
  uint8_t e = 1;
  for (int v = 0; v < 3; v++) e = hf::f8_mul(e, ((xs >> v) & 1) ? SMALL_CHAL[v] : (uint8_t)(1 ^ SMALL_CHAL[v]));
  return e;
}

// eq weight of r7, r8 only (variables 1, 2 of xs), for the c statistic.
inline uint8_t e8c(int x2) {
  uint8_t e = 1;
  for (int v = 1; v < 3; v++) e = hf::f8_mul(e, ((x2 >> (v - 1)) & 1) ? SMALL_CHAL[v] : (uint8_t)(1 ^ SMALL_CHAL[v]));
  return e;
}

inline void build_round1_tables(ZcRound1Tables& T) {
  for (int x2 = 0; x2 < 4; x2++) T.e8c[x2] = e8c(x2);
  auto M = ext_matrix();
  for (int c = 0; c < 8; c++)
    for (int v = 0; v < 256; v++) {
      uint64_t pl[8] = {0};
      for (int i = 0; i < 64; i++) {
        uint8_t val = 0;
        for (int t = 0; t < 8; t++)
          if ((v >> t) & 1) val ^= M[i * 64 + 8 * c + t];
        for (int j = 0; j < 8; j++)
          if ((val >> j) & 1) pl[j] |= 1ULL << i;
      }
      for (int j = 0; j < 8; j++) T.ext[c][v][j] = pl[j];
    }
  for (int v = 0; v < 256; v++) {
    hf::F p = hf::phi8((uint8_t)v);
    T.phi8[v][0] = p.lo;
    T.phi8[v][1] = p.hi;
  }
  for (int xs = 0; xs < 8; xs++) {
    T.e8[xs] = e8(xs);
  }
}

// Dinv = prod_j (1 + x^(2^j))^-1, the constant of the four medium challenges.
inline hf::F medium_dinv() {
  hf::F d = hf::F::one();
  for (int j = 0; j < 4; j++) d = d * (hf::F::one() + hf::F(1ULL << (1 << j), 0));
  return hf::inv(d);
}

}  // namespace zc

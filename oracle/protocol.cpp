// Oracle restatement of the Flock R1CS prover and verifier (test infrastructure only).
//
// Follows, in order: bind_statement (crates/flock-core/src/proof.rs:51-59),
// zerocheck (crates/flock-core/src/zerocheck.rs:482-1360, naive forms in
// zerocheck/univariate_skip.rs:84-138 and zerocheck/multilinear.rs:361-675,
// verifier :1365-1517), lincheck (crates/flock-core/src/lincheck.rs:1480-1840),
// ring switch (crates/flock-core/src/pcs/ring_switch.rs:2708-3450,
// crates/flock-core/src/pcs.rs:1025-1110, :1719-1858) and the recursive
// Ligerito PCS (crates/flock-core/src/pcs/ligerito.rs:1673-2160, :3340-3557,
// :3672-3780, :5367-5850, :6222-6980 prover, :6981-7545 verifier).
// Every message is computed from its defining formula, so the proof bytes are
// the unique ones the reference's optimized prover must also emit.
#include "protocol.h"

#include <algorithm>
#include <cstring>
#include <set>
#include <stdexcept>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

static inline F128 one() { return f128(1); }

// ============================================================================
// Transcript
// ============================================================================
static void le64(uint64_t v, uint8_t b[8]) {
  for (int i = 0; i < 8; i++) b[i] = (uint8_t)(v >> (8 * i));
}

Transcript::Transcript(const std::string& domain) {
  uint8_t op = 0x01, len[8];
  le64(domain.size(), len);
  absorb(&op, 1);
  absorb(len, 8);
  absorb(domain.data(), domain.size());
}
void Transcript::label(const std::string& s) {
  uint8_t op = 0x02, len[8];
  le64(s.size(), len);
  absorb(&op, 1);
  absorb(len, 8);
  absorb(s.data(), s.size());
}
void Transcript::observe_f128(F128 v) {
  uint8_t b[18] = {0x03, 0x01};
  le64(v.lo, b + 2);
  le64(v.hi, b + 10);
  absorb(b, 18);
}
void Transcript::observe_slice(const F128* v, size_t n) {
  uint8_t b[10] = {0x03, 0x02};
  le64(n, b + 2);
  absorb(b, 10);
  absorb(v, 16 * n);  // little-endian lo||hi per element
}
void Transcript::observe_bytes(const uint8_t* p, size_t n) {
  uint8_t b[9] = {0x05};
  le64(n, b + 1);
  absorb(b, 9);
  absorb(p, n);
}
F128 Transcript::sample() {
  uint8_t op[2] = {0x04, 0x01};
  absorb(op, 2);
  uint8_t buf[16];
  h.finalize_xof(buf, 16);
  absorb(buf, 16);
  F128 r;
  memcpy(&r.lo, buf, 8);
  memcpy(&r.hi, buf + 8, 8);
  return r;
}
std::vector<F128> Transcript::sample_vec(size_t n) {
  uint8_t b[10] = {0x04, 0x02};
  le64(n, b + 2);
  absorb(b, 10);
  std::vector<F128> out(n);
  if (n) {
    h.finalize_xof((uint8_t*)out.data(), 16 * n);
    absorb(out.data(), 16 * n);
  }
  return out;
}
void Transcript::state_digest(uint8_t out[32]) const { h.finalize(out); }

// challenger.rs:1246-1296: BLAKE3 of digest || nonce_le || 0^24 (one 64-byte
// root block), at least `bits` leading zero bits, byte-wise MSB first.
bool pow_ok(const uint8_t digest[32], uint64_t nonce, uint32_t bits) {
  uint8_t pre[64] = {0};
  memcpy(pre, digest, 32);
  le64(nonce, pre + 32);
  uint8_t hsh[32];
  b3_hash(pre, 64, hsh);
  uint32_t full = bits / 8, extra = bits % 8;
  for (uint32_t i = 0; i < full; i++)
    if (hsh[i]) return false;
  if (extra && (hsh[full] >> (8 - extra))) return false;
  return true;
}

uint64_t Transcript::grind(uint32_t bits) {
  uint64_t nonce = 0;
  if (bits > 0) {
    uint8_t d[32];
    state_digest(d);
    // Smallest satisfying nonce: scan blocks in parallel, keep the minimum.
    const uint64_t BLOCK = 1 << 16;
    for (uint64_t start = 0;; start += BLOCK) {
      uint64_t best = UINT64_MAX;
#pragma omp parallel for reduction(min : best) schedule(static)
      for (int64_t i = 0; i < (int64_t)BLOCK; i++)
        if (pow_ok(d, start + (uint64_t)i, bits)) best = std::min(best, start + (uint64_t)i);
      if (best != UINT64_MAX) { nonce = best; break; }
    }
  }
  uint8_t b[8];
  le64(nonce, b);
  observe_bytes(b, 8);
  return nonce;
}
bool Transcript::verify_pow(uint64_t nonce, uint32_t bits) {
  uint8_t d[32];
  state_digest(d);
  bool ok = bits == 0 ? nonce == 0 : pow_ok(d, nonce, bits);
  uint8_t b[8];
  le64(nonce, b);
  observe_bytes(b, 8);
  return ok;
}

// ============================================================================
// Helpers
// ============================================================================
std::vector<F128> eq_table(const std::vector<F128>& r) {
  std::vector<F128> t((size_t)1 << r.size());
  t[0] = one();
  for (size_t i = 0; i < r.size(); i++) {
    size_t half = (size_t)1 << i;
#pragma omp parallel for if (half > 4096)
    for (int64_t j = 0; j < (int64_t)half; j++) {
      F128 v = t[j], vr = v * r[i];
      t[j + half] = vr;
      t[j] = v + vr;
    }
  }
  return t;
}

static std::vector<F128> lagrange_nodes(F128 z, int off, int n) {
  // multilinear.rs:361-470 reference loop: prod_{j!=i}(z+s_j) / prod_{j!=i}(s_i+s_j)
  std::vector<F128> w(n);
  for (int i = 0; i < n; i++) {
    F128 si = phi8((uint8_t)(off + i)), num = one(), den = one();
    for (int j = 0; j < n; j++) {
      if (j == i) continue;
      F128 sj = phi8((uint8_t)(off + j));
      num = num * (z + sj);
      den = den * (si + sj);
    }
    w[i] = num * gf_inv(den);
  }
  return w;
}
std::vector<F128> lagrange_s(F128 z) { return lagrange_nodes(z, 0, 64); }
std::vector<F128> lagrange_lambda(F128 z) { return lagrange_nodes(z, 64, 64); }

static F128 interpolate_lambda(const std::vector<F128>& v, F128 z) {
  auto w = lagrange_lambda(z);
  F128 acc;
  for (int i = 0; i < 64; i++) acc += w[i] * v[i];
  return acc;
}
// multilinear.rs:522-548
F128 interpolate_combined(const std::vector<F128>& on_lambda, F128 z) {
  F128 acc;
  for (int i = 0; i < 64; i++) {
    int node = 64 + i;
    F128 si = phi8((uint8_t)node), num = one(), den = one();
    for (int j = 0; j < 128; j++) {
      if (j == node) continue;
      F128 sj = phi8((uint8_t)j);
      num = num * (z + sj);
      den = den * (si + sj);
    }
    acc += num * gf_inv(den) * on_lambda[i];
  }
  return acc;
}

static F128 dot(const F128* a, const F128* b, size_t n) {
  F128 acc;
  for (size_t i = 0; i < n; i++) acc += a[i] * b[i];
  return acc;
}

// F8 additive NTT, crates/flock-core/src/ntt.rs:25-170.
static uint8_t f8_next_s(uint8_t s, uint8_t root) { return gf8_mul(s, s) ^ gf8_mul(root, s); }
static std::vector<uint8_t> f8_twiddles(int k, uint8_t beta) {
  size_t n = (size_t)1 << k;
  std::vector<uint8_t> tw(n - 1);
  size_t len = n >> 1;
  std::vector<uint8_t> layer(len);
  for (size_t i = 0; i < len; i++) layer[i] = beta ^ (uint8_t)(2 * i);
  uint8_t s_root = 1;
  size_t write_at = len;
  for (size_t i = 0; i < len; i++) tw[write_at - 1 + i] = layer[i];
  for (int it = 1; it < k; it++) {
    write_at >>= 1;
    uint8_t next_root = f8_next_s(layer[1] ^ layer[0], s_root);
    size_t new_len = write_at;
    for (size_t i = 0; i < new_len; i++) layer[i] = f8_next_s(layer[2 * i], s_root);
    len = new_len;
    s_root = next_root;
    uint8_t inv = gf8_inv(s_root);
    for (size_t j = 0; j < len; j++) tw[write_at - 1 + j] = gf8_mul(inv, layer[j]);
  }
  return tw;
}
static void f8_fft_rec(uint8_t* v, size_t n, const uint8_t* tw, size_t idx) {
  if (n == 1) return;
  size_t half = n / 2;
  uint8_t lam = tw[idx - 1];
  for (size_t i = 0; i < half; i++) {
    uint8_t w = v[half + i];
    v[i] ^= gf8_mul(lam, w);
    v[half + i] = w ^ v[i];
  }
  f8_fft_rec(v, half, tw, 2 * idx);
  f8_fft_rec(v + half, half, tw, 2 * idx + 1);
}
static void f8_ifft_rec(uint8_t* v, size_t n, const uint8_t* tw, size_t idx) {
  if (n == 1) return;
  size_t half = n / 2;
  f8_ifft_rec(v, half, tw, 2 * idx);
  f8_ifft_rec(v + half, half, tw, 2 * idx + 1);
  uint8_t lam = tw[idx - 1];
  for (size_t i = 0; i < half; i++) {
    v[half + i] ^= v[i];
    v[i] ^= gf8_mul(lam, v[half + i]);
  }
}
void f8_ntt_forward(uint8_t* v, int k, uint8_t beta) {
  auto tw = f8_twiddles(k, beta);
  f8_fft_rec(v, (size_t)1 << k, tw.data(), 1);
}
void f8_ntt_inverse(uint8_t* v, int k, uint8_t beta) {
  auto tw = f8_twiddles(k, beta);
  f8_ifft_rec(v, (size_t)1 << k, tw.data(), 1);
}

// ============================================================================
// Zerocheck
// ============================================================================
struct ZcClaim {
  F128 z;
  std::vector<F128> mlv, r_rest;
  F128 a_eval, b_eval, c_eval;
};

static std::vector<F128> zc_challenges(Transcript& tr, int m) {
  // zerocheck.rs:509-532 (prover) / :1400-1412 (verifier)
  auto r_skip = tr.sample_vec(6);
  auto r_outer = tr.sample_vec(m - 13);
  std::vector<F128> r(m);
  for (int i = 0; i < 6; i++) r[i] = r_skip[i];
  // univariate_skip_optimized.rs:85-120: phi8(0xF7,0x53,0xB5), then g/(1+g), g = x^(2^i)
  const uint8_t small[3] = {0xF7, 0x53, 0xB5};
  for (int i = 0; i < 3; i++) r[6 + i] = phi8(small[i]);
  for (int i = 0; i < 4; i++) {
    F128 g = f128(1ULL << (1 << i));
    r[9 + i] = g * gf_inv(one() + g);
  }
  for (int i = 13; i < m; i++) r[i] = r_outer[i - 13];
  return r;
}

// F8 Lagrange extension S = {0..63} -> Lambda = {64..127}, as byte tables over
// the 8 bytes of a 64-bit row: TL[c][v][i] = ext(bits of v at s = 8c..8c+7)(lambda_i).
struct ExtTables {
  uint8_t t[8][256][64];
  uint8_t exp[512], log[256];
  ExtTables() {
    uint8_t M[64][64];
    for (int i = 0; i < 64; i++)
      for (int s = 0; s < 64; s++) {
        uint8_t num = 1, den = 1, lam = (uint8_t)(64 + i);
        for (int t2 = 0; t2 < 64; t2++) {
          if (t2 == s) continue;
          num = gf8_mul(num, lam ^ (uint8_t)t2);
          den = gf8_mul(den, (uint8_t)(s ^ t2));
        }
        M[i][s] = gf8_mul(num, gf8_inv(den));
      }
    for (int c = 0; c < 8; c++)
      for (int v = 0; v < 256; v++)
        for (int i = 0; i < 64; i++) {
          uint8_t acc = 0;
          for (int j = 0; j < 8; j++)
            if ((v >> j) & 1) acc ^= M[i][8 * c + j];
          t[c][v][i] = acc;
        }
    uint8_t x = 1;
    for (int i = 0; i < 255; i++) {
      exp[i] = exp[i + 255] = x;
      log[x] = (uint8_t)i;
      x = gf8_mul(x, 3);
    }
    exp[510] = exp[0];
    exp[511] = exp[1];
    log[0] = 0;
  }
  void ext(uint64_t w, uint8_t out[64]) const {
    memset(out, 0, 64);
    for (int c = 0; c < 8; c++) {
      const uint8_t* row = t[c][(w >> (8 * c)) & 255];
      for (int i = 0; i < 64; i++) out[i] ^= row[i];
    }
  }
  uint8_t mul(uint8_t a, uint8_t b) const { return (a && b) ? exp[log[a] + log[b]] : 0; }
};
static const ExtTables& ext_tables() {
  static const ExtTables t;
  return t;
}

static inline uint64_t tr8(uint64_t x) {
  uint64_t t;
  t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAULL; x = x ^ t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCULL; x = x ^ t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ULL; x = x ^ t ^ (t << 28);
  return x;
}

// P^AB(lambda_i) and P^C(lambda_i) of univariate_skip.rs:84-138 (naive
// convention): sum_x eq(r_rest, x) * phi8(a^(l,x) b^(l,x)) and phi8(c^(l,x)).
static void zc_round1(const uint64_t* A, const uint64_t* B, const uint64_t* C, size_t rows,
                      const std::vector<F128>& eq, std::vector<F128>& pab, std::vector<F128>& pc) {
  const ExtTables& T = ext_tables();
  std::vector<F128> acc_ab(512), acc_c(512);
#pragma omp parallel
  {
    std::vector<F128> lab(512), lc(512);
    F128 t8[256];
#pragma omp for schedule(static)
    for (int64_t g = 0; g < (int64_t)(rows / 8); g++) {
      size_t x0 = (size_t)g * 8;
      t8[0] = F128();
      for (int v = 1; v < 256; v++) {
        int low = __builtin_ctz(v);
        t8[v] = t8[v & (v - 1)] + eq[x0 + low];
      }
      uint8_t y[8][64], cc[8][64];
      for (int r = 0; r < 8; r++) {
        uint8_t ea[64], eb[64];
        T.ext(A[x0 + r], ea);
        T.ext(B[x0 + r], eb);
        T.ext(C[x0 + r], cc[r]);
        for (int i = 0; i < 64; i++) y[r][i] = T.mul(ea[i], eb[i]);
      }
      for (int i = 0; i < 64; i++) {
        uint64_t xa = 0, xc = 0;
        for (int r = 0; r < 8; r++) {
          xa |= (uint64_t)y[r][i] << (8 * r);
          xc |= (uint64_t)cc[r][i] << (8 * r);
        }
        xa = tr8(xa);
        xc = tr8(xc);
        for (int k = 0; k < 8; k++) {
          lab[i * 8 + k] += t8[(xa >> (8 * k)) & 255];
          lc[i * 8 + k] += t8[(xc >> (8 * k)) & 255];
        }
      }
    }
#pragma omp critical
    for (int j = 0; j < 512; j++) {
      acc_ab[j] += lab[j];
      acc_c[j] += lc[j];
    }
  }
  pab.assign(64, F128());
  pc.assign(64, F128());
  for (int i = 0; i < 64; i++)
    for (int k = 0; k < 8; k++) {
      F128 p = phi8((uint8_t)(1 << k));
      pab[i] += p * acc_ab[i * 8 + k];
      pc[i] += p * acc_c[i * 8 + k];
    }
}

// Fold each 64-bit row at the skip point: out[x] = sum_s bit_s(w_x) L_s(z).
static std::vector<F128> fold_skip(const uint64_t* W, size_t rows, const std::vector<F128>& L) {
  std::vector<F128> tab(8 * 256);
  for (int c = 0; c < 8; c++)
    for (int v = 0; v < 256; v++) {
      F128 acc;
      for (int j = 0; j < 8; j++)
        if ((v >> j) & 1) acc += L[8 * c + j];
      tab[c * 256 + v] = acc;
    }
  std::vector<F128> out(rows);
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < (int64_t)rows; x++) {
    F128 acc;
    for (int c = 0; c < 8; c++) acc += tab[c * 256 + ((W[x] >> (8 * c)) & 255)];
    out[x] = acc;
  }
  return out;
}

static ZerocheckProof zc_prove(const uint64_t* A, const uint64_t* B, const uint64_t* C, int m, Transcript& tr,
                               ZcClaim& claim) {
  ZerocheckProof pf;
  tr.label("flock-zerocheck-v0");
  auto r = zc_challenges(tr, m);
  size_t rows = (size_t)1 << (m - 6);
  {
    std::vector<F128> rr(r.begin() + 6, r.end());
    auto eq = eq_table(rr);
    zc_round1(A, B, C, rows, eq, pf.round1_ab, pf.round1_c);
  }
  tr.observe_slice(pf.round1_ab.data(), 64);
  tr.observe_slice(pf.round1_c.data(), 64);
  F128 z = tr.sample();
  pf.final_c = interpolate_lambda(pf.round1_c, z);
  auto L = lagrange_s(z);
  auto fa = fold_skip(A, rows, L);
  auto fb = fold_skip(B, rows, L);
  int n_mlv = m - 6;
  std::vector<F128> rho;
  for (int i = 0; i < n_mlv; i++) {
    size_t half = fa.size() / 2;
    std::vector<F128> rr(r.begin() + 6 + i + 1, r.end());
    auto eq = eq_table(rr);
    F128 g1, ginf;
#pragma omp parallel
    {
      F128 l1, li;
#pragma omp for schedule(static)
      for (int64_t j = 0; j < (int64_t)half; j++) {
        F128 a0 = fa[2 * j], a1 = fa[2 * j + 1], b0 = fb[2 * j], b1 = fb[2 * j + 1];
        l1 += eq[j] * (a1 * b1);
        li += eq[j] * ((a0 + a1) * (b0 + b1));
      }
#pragma omp critical
      {
        g1 += l1;
        ginf += li;
      }
    }
    pf.rounds.push_back({g1, ginf});
    tr.observe_f128(g1);
    tr.observe_f128(ginf);
    F128 p = tr.sample();
    rho.push_back(p);
    std::vector<F128> na(half), nb(half);
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < (int64_t)half; j++) {
      na[j] = fa[2 * j] + p * (fa[2 * j] + fa[2 * j + 1]);
      nb[j] = fb[2 * j] + p * (fb[2 * j] + fb[2 * j + 1]);
    }
    fa.swap(na);
    fb.swap(nb);
  }
  pf.final_a = fa[0];
  pf.final_b = fb[0];
  tr.observe_f128(pf.final_a);
  tr.observe_f128(pf.final_b);
  claim.z = z;
  claim.mlv = rho;
  claim.r_rest.assign(r.begin() + 6, r.end());
  claim.a_eval = pf.final_a;
  claim.b_eval = pf.final_b;
  claim.c_eval = pf.final_c;
  return pf;
}

static bool zc_verify(const ZerocheckProof& pf, int m, Transcript& tr, ZcClaim& claim, std::string* why) {
  int n_mlv = m - 6;
  if (pf.round1_ab.size() != 64 || pf.round1_c.size() != 64 || (int)pf.rounds.size() != n_mlv) {
    if (why) *why = "zerocheck shape";
    return false;
  }
  tr.label("flock-zerocheck-v0");
  auto r = zc_challenges(tr, m);
  tr.observe_slice(pf.round1_ab.data(), 64);
  tr.observe_slice(pf.round1_c.data(), 64);
  F128 z = tr.sample();
  if (interpolate_lambda(pf.round1_c, z) != pf.final_c) {
    if (why) *why = "zerocheck c-eval";
    return false;
  }
  std::vector<F128> comb(64);
  for (int i = 0; i < 64; i++) comb[i] = pf.round1_ab[i] + pf.round1_c[i];
  F128 running = interpolate_combined(comb, z) + interpolate_lambda(pf.round1_c, z);
  std::vector<F128> rho;
  for (int i = 0; i < n_mlv; i++) {
    F128 req = r[6 + i], g1 = pf.rounds[i].first, gi = pf.rounds[i].second;
    F128 g0 = (running + req * g1) * gf_inv(one() + req);
    tr.observe_f128(g1);
    tr.observe_f128(gi);
    F128 p = tr.sample();
    rho.push_back(p);
    F128 op = one() + p;
    running = g0 * op + g1 * p + gi * p * op;
  }
  if (running != pf.final_a * pf.final_b) {
    if (why) *why = "zerocheck sumcheck final";
    return false;
  }
  tr.observe_f128(pf.final_a);
  tr.observe_f128(pf.final_b);
  claim.z = z;
  claim.mlv = rho;
  claim.r_rest.assign(r.begin() + 6, r.end());
  claim.a_eval = pf.final_a;
  claim.b_eval = pf.final_b;
  claim.c_eval = pf.final_c;
  return true;
}

// ============================================================================
// Lincheck
// ============================================================================
struct LcClaim {
  F128 r_inner_skip, w;
  std::vector<F128> r_inner_rest;
};

// lincheck.rs:1127-1143: index i_skip + 64 * i_rest.
static std::vector<F128> quirky_eq(F128 z_skip, const std::vector<F128>& x_inner_rest) {
  auto L = lagrange_s(z_skip);
  auto e = eq_table(x_inner_rest);
  std::vector<F128> out;
  out.reserve(64 * e.size());
  for (auto& er : e)
    for (auto& ls : L) out.push_back(ls * er);
  return out;
}

// alpha * A0^T eq + B0^T eq (lincheck.rs:1160-1240 sparse fold), + beta at the pin.
static std::vector<F128> lc_comb(const SparseRows& A, const SparseRows& B, F128 alpha, F128 beta,
                                 const std::vector<F128>& eq) {
  std::vector<F128> comb(K);
  for (int r = 0; r < K; r++) {
    if (eq[r].is_zero()) continue;
    F128 ae = alpha * eq[r];
    for (uint32_t c : A.rows[r]) comb[c] += ae;
    for (uint32_t c : B.rows[r]) comb[c] += eq[r];
  }
  comb[Z_CONST_POS] += beta;
  return comb;
}

static void bind_top(std::vector<F128>& v, F128 r) {
  size_t half = v.size() / 2;
  for (size_t i = 0; i < half; i++) v[i] = v[i] + r * (v[i + half] + v[i]);
  v.resize(half);
}

static LincheckProof lc_prove(const uint8_t* stripe, int m, const SparseRows& A, const SparseRows& B, F128 z_skip,
                              const std::vector<F128>& x_inner_rest, const std::vector<F128>& x_outer,
                              Transcript& tr, LcClaim& claim) {
  LincheckProof pf;
  tr.label("flock-lincheck-v0");
  F128 alpha = tr.sample();
  F128 beta = tr.sample();
  auto eq_in = quirky_eq(z_skip, x_inner_rest);
  auto comb = lc_comb(A, B, alpha, beta, eq_in);
  // z_vec[i_inner] = sum_outer z[i_inner, outer] eq(x_outer)[outer] (lincheck.rs:655-690)
  auto eq_out = eq_table(x_outer);
  size_t n_stripes = eq_out.size() / 8;
  std::vector<F128> zv(K);
#pragma omp parallel
  {
    std::vector<F128> loc(K);
    F128 t8[256];
#pragma omp for schedule(static)
    for (int64_t s = 0; s < (int64_t)n_stripes; s++) {
      t8[0] = F128();
      for (int v = 1; v < 256; v++) t8[v] = t8[v & (v - 1)] + eq_out[8 * s + __builtin_ctz(v)];
      const uint8_t* row = stripe + (size_t)s * K;
      for (int i = 0; i < K; i++)
        if (row[i]) loc[i] += t8[row[i]];
    }
#pragma omp critical
    for (int i = 0; i < K; i++) zv[i] += loc[i];
  }
  std::vector<F128> rr;
  for (int t = 0; t < K_LOG - K_SKIP; t++) {
    size_t half = comb.size() / 2;
    F128 e1, ei;
    for (size_t i = 0; i < half; i++) {
      e1 += comb[i + half] * zv[i + half];
      ei += (comb[i + half] + comb[i]) * (zv[i + half] + zv[i]);
    }
    tr.observe_f128(e1);
    tr.observe_f128(ei);
    F128 r = tr.sample();
    pf.rounds.push_back({e1, ei});
    rr.push_back(r);
    bind_top(comb, r);
    bind_top(zv, r);
  }
  pf.z_partial = zv;
  tr.observe_slice(zv.data(), zv.size());
  claim.r_inner_skip = tr.sample();
  auto L = lagrange_s(claim.r_inner_skip);
  claim.w = dot(L.data(), zv.data(), 64);
  claim.r_inner_rest.assign(rr.rbegin(), rr.rend());
  return pf;
}

static bool lc_verify(const LincheckProof& pf, const SparseRows& A, const SparseRows& B, F128 z_skip,
                      const std::vector<F128>& x_inner_rest, F128 va, F128 vb, Transcript& tr, LcClaim& claim,
                      std::string* why) {
  if ((int)pf.rounds.size() != K_LOG - K_SKIP || pf.z_partial.size() != 64) {
    if (why) *why = "lincheck shape";
    return false;
  }
  tr.label("flock-lincheck-v0");
  F128 alpha = tr.sample();
  auto eq_in = quirky_eq(z_skip, x_inner_rest);
  F128 beta = tr.sample();
  auto comb = lc_comb(A, B, alpha, beta, eq_in);
  F128 running = alpha * va + vb + beta;
  std::vector<F128> rr;
  for (auto& rd : pf.rounds) {
    tr.observe_f128(rd.first);
    tr.observe_f128(rd.second);
    F128 r = tr.sample();
    F128 e0 = running + rd.first;
    F128 c1 = e0 + rd.first + rd.second;
    running = rd.second * r * r + c1 * r + e0;
    bind_top(comb, r);
    rr.push_back(r);
  }
  tr.observe_slice(pf.z_partial.data(), 64);
  if (dot(comb.data(), pf.z_partial.data(), 64) != running) {
    if (why) *why = "lincheck final";
    return false;
  }
  claim.r_inner_skip = tr.sample();
  auto L = lagrange_s(claim.r_inner_skip);
  claim.w = dot(L.data(), pf.z_partial.data(), 64);
  claim.r_inner_rest.assign(rr.rbegin(), rr.rend());
  return true;
}

// ============================================================================
// Ring switch (ring_switch.rs:1568-1760, :2708-2780)
// ============================================================================
static std::vector<F128> fold_1b_rows(const std::vector<F128>& z, const std::vector<F128>& t) {
  std::vector<F128> acc(16 * 256);
#pragma omp parallel
  {
    std::vector<F128> loc(16 * 256);
#pragma omp for schedule(static)
    for (int64_t p = 0; p < (int64_t)z.size(); p++) {
      const uint8_t* by = (const uint8_t*)&z[p];
      for (int q = 0; q < 16; q++)
        if (by[q]) loc[q * 256 + by[q]] += t[p];
    }
#pragma omp critical
    for (int i = 0; i < 16 * 256; i++) acc[i] += loc[i];
  }
  std::vector<F128> s(128);
  for (int q = 0; q < 16; q++)
    for (int v = 1; v < 256; v++)
      for (int j = 0; j < 8; j++)
        if ((v >> j) & 1) s[8 * q + j] += acc[q * 256 + v];
  return s;
}
static std::vector<F128> transpose128(const std::vector<F128>& v) {
  std::vector<F128> u(128);
  for (int i = 0; i < 128; i++)
    for (int b = 0; b < 128; b++) {
      uint64_t bit = b < 64 ? (v[i].lo >> b) & 1 : (v[i].hi >> (b - 64)) & 1;
      if (bit) {
        if (i < 64) u[b].lo |= 1ULL << i;
        else u[b].hi |= 1ULL << (i - 64);
      }
    }
  return u;
}
static std::vector<F128> fold_b128(const std::vector<F128>& t, const std::vector<F128>& eqr) {
  std::vector<F128> tab(16 * 256);
  for (int q = 0; q < 16; q++)
    for (int v = 1; v < 256; v++) tab[q * 256 + v] = tab[q * 256 + (v & (v - 1))] + eqr[8 * q + __builtin_ctz(v)];
  std::vector<F128> out(t.size());
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < (int64_t)t.size(); p++) {
    const uint8_t* by = (const uint8_t*)&t[p];
    F128 acc;
    for (int q = 0; q < 16; q++) acc += tab[q * 256 + by[q]];
    out[p] = acc;
  }
  return out;
}
// ring_switch.rs:138-157
static std::vector<F128> claim_weights(F128 z_skip, F128 x0) {
  auto L = lagrange_s(z_skip);
  std::vector<F128> w(128);
  for (int i = 0; i < 128; i++) w[i] = L[i & 63] * ((i >> 6) & 1 ? x0 : one() + x0);
  return w;
}

// ============================================================================
// Ligerito
// ============================================================================
bool ligerito_config(int m, int profile, LigConfig& c) {
// the parameter table generated from the reference TOMLs, shared with the product library
#include "../flock_challenge_gb300/csrc/ligerito_params.inc"
  for (int i = 0; i < LIGERITO_N_CONFIGS; i++) {
    const int* row = LIGERITO_CONFIGS[i];
    if (row[0] != m || row[1] != profile) continue;
    c = LigConfig();
    c.initial_k = row[2];
    c.yr_log_n = row[3];
    int nl = row[4];
    c.steps = nl - 1;
    for (int l = 0; l < nl; l++) {
      const int* L = row + 5 + 8 * l;
      c.log_inv_rates.push_back(L[0]);
      if (l > 0) c.ks.push_back(L[3]);
      c.queries.push_back(L[4]);
      c.grinding_bits.push_back(L[5]);
      c.fold_bits.push_back(L[6]);
      c.ood.push_back(L[7]);
    }
    return true;
  }
  return false;
}

static int ceil_log2(size_t n) {
  int l = 0;
  while (((size_t)1 << l) < n) l++;
  return l;
}

struct Msg {
  F128 u0, u2;
};
static Msg round_msg(const std::vector<F128>& f, const std::vector<F128>& b, F128* h = nullptr) {
  size_t half = f.size() / 2;
  F128 u0, u2, hh;
#pragma omp parallel
  {
    F128 l0, l2, lh;
#pragma omp for schedule(static)
    for (int64_t j = 0; j < (int64_t)half; j++) {
      F128 f0 = f[2 * j], f1 = f[2 * j + 1], b0 = b[2 * j], b1 = b[2 * j + 1];
      l0 += f0 * b0;
      l2 += (f0 + f1) * (b0 + b1);
      if (h) lh += f0 * b0 + f1 * b1;
    }
#pragma omp critical
    {
      u0 += l0;
      u2 += l2;
      hh += lh;
    }
  }
  if (h) *h = hh;
  return {u0, u2};
}
static void fold_lsb(std::vector<F128>& v, F128 r) {
  size_t half = v.size() / 2;
  for (size_t j = 0; j < half; j++) v[j] = v[2 * j] + r * (v[2 * j] + v[2 * j + 1]);
  v.resize(half);
}

struct LigeroWitness {
  std::vector<F128> mat;
  std::vector<Hash32> tree;
  size_t block_len = 0, ni = 0;
};
static LigeroWitness ligero_commit(const std::vector<F128>& poly, int log_msg_cols, int log_ni, int rate) {
  LigeroWitness w;
  w.ni = (size_t)1 << log_ni;
  w.block_len = (size_t)1 << (log_msg_cols + rate);
  w.mat.resize(w.block_len * w.ni);
  for (size_t i = 0; i < w.mat.size(); i++) w.mat[i] = poly[i % poly.size()];
  NttF128 ntt(log_msg_cols + rate);
  ntt.forward_interleaved(w.mat.data(), w.mat.size(), w.ni, rate);
  w.tree = merkle_tree((const uint8_t*)w.mat.data(), w.mat.size() * 16, w.block_len);
  return w;
}

static std::vector<size_t> sample_queries(Transcript& tr, size_t block_len, size_t count) {
  std::set<size_t> seen;
  std::vector<size_t> out;
  while (out.size() < count) {
    F128 v = tr.sample();
    size_t q = (size_t)(v.lo % block_len);
    if (seen.insert(q).second) out.push_back(q);
  }
  std::sort(out.begin(), out.end());
  return out;
}

// ligerito.rs:1747-1774
static std::vector<F128> sk_at_vk(int n) {
  std::vector<F128> s(n + 1);
  s[0] = one();
  if (n == 0) return s;
  std::vector<F128> layer;
  for (int i = 1; i <= n; i++) layer.push_back(f128(1ULL << i));
  int cur = n;
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < cur; j++) {
      F128 v = layer[j] * layer[j] + s[i] * layer[j];
      if (j == 0) s[i + 1] = v;
      else layer[j - 1] = v;
    }
    cur--;
  }
  return s;
}
// Normalized What_k(q) for k < n (ligerito.rs:1776-1824).
static std::vector<F128> what_at(int n, const std::vector<F128>& sks, size_t q) {
  std::vector<F128> w(n);
  if (n == 0) return w;
  w[0] = f128(q);
  for (int i = 1; i < n; i++) w[i] = w[i - 1] * w[i - 1] + sks[i - 1] * w[i - 1];
  for (int i = 0; i < n; i++) w[i] = w[i] * gf_inv(sks[i]);
  return w;
}

// ligerito.rs:1989-2160: basis[j] = sum_i alpha_i Xhat_j(q_i); enforced = sum_i alpha_i <row_i, eq(v)>.
static void induce(int n, const std::vector<std::vector<F128>>& rows, const std::vector<F128>& v,
                   const std::vector<size_t>& queries, const std::vector<F128>& alpha, std::vector<F128>& basis,
                   F128& enforced) {
  auto sks = sk_at_vk(n);
  auto eqv = eq_table(v);
  auto at = eq_table(alpha);
  basis.assign((size_t)1 << n, F128());
  enforced = F128();
  std::vector<F128> loc((size_t)1 << n);
  for (size_t i = 0; i < queries.size(); i++) {
    enforced += at[i] * dot(rows[i].data(), eqv.data(), rows[i].size());
    auto w = what_at(n, sks, queries[i]);
    loc[0] = at[i];
    for (int k = 0; k < n; k++) {
      size_t len = (size_t)1 << k;
      for (size_t j = 0; j < len; j++) loc[j + len] = w[k] * loc[j];
    }
    for (size_t j = 0; j < loc.size(); j++) basis[j] += loc[j];
  }
}

static LevelOpen open_rows(const LigeroWitness& w, const std::vector<size_t>& q) {
  LevelOpen o;
  for (size_t p : q) o.rows.emplace_back(w.mat.begin() + p * w.ni, w.mat.begin() + (p + 1) * w.ni);
  o.proof = merkle_multi_proof(w.tree, w.block_len, q);
  return o;
}

struct SumcheckProver {
  std::vector<F128> f, basis, pend;
  bool has_pend = false;
  std::vector<std::pair<F128, F128>> msgs;
  Msg push(Msg m) {
    msgs.push_back({m.u0, m.u2});
    return m;
  }
  Msg fold(F128 r) {
    fold_lsb(f, r);
    fold_lsb(basis, r);
    return push(round_msg(f, basis));
  }
  Msg introduce(std::vector<F128> b) {
    Msg m = round_msg(f, b);
    pend = std::move(b);
    has_pend = true;
    return push(m);
  }
  Msg introduce_eval(std::vector<F128> b, F128& h) {
    Msg m = round_msg(f, b, &h);
    pend = std::move(b);
    has_pend = true;
    return push(m);
  }
  void glue(F128 beta) {
    for (size_t i = 0; i < basis.size(); i++) basis[i] += beta * pend[i];
    pend.clear();
    has_pend = false;
  }
};

static LigeritoProof ligerito_prove(const LigConfig& cfg, std::vector<F128> f, std::vector<F128> b, F128 target,
                                    const CommitData& l0, Transcript& tr) {
  LigeritoProof pf;
  int log_n = ceil_log2(f.size());
  int k0 = cfg.initial_k;
  size_t block0 = (size_t)1 << (log_n - k0 + cfg.log_inv_rates[0]);
  size_t ni0 = (size_t)1 << k0;
  tr.label("flock-ligerito-basis-v0");
  tr.observe_f128(target);
  pf.initial_root = l0.root();
  tr.observe_bytes(pf.initial_root.b, 32);
  SumcheckProver sc;
  sc.f = std::move(f);
  sc.basis = std::move(b);
  Msg m0 = sc.push(round_msg(sc.f, sc.basis));
  tr.observe_f128(m0.u0);
  tr.observe_f128(m0.u2);
  auto fb = [&](int lvl) { return (uint32_t)(lvl < (int)cfg.fold_bits.size() ? cfg.fold_bits[lvl] : 0); };
  auto ood = [&](int lvl) { return lvl < (int)cfg.ood.size() ? cfg.ood[lvl] : 0; };
  std::vector<F128> r_lane;
  for (int j = 0; j < k0; j++) {
    uint32_t bits = fb(0) > (uint32_t)j ? fb(0) - j : 0;
    if (bits) pf.fold_nonces.push_back(tr.grind(bits));
    F128 r = tr.sample();
    Msg m = sc.fold(r);
    tr.observe_f128(m.u0);
    tr.observe_f128(m.u2);
    r_lane.push_back(r);
  }
  int n1 = log_n - k0;
  int lni1 = cfg.ks[0];
  LigeroWitness wprev = ligero_commit(sc.f, n1 - lni1, lni1, cfg.log_inv_rates[1]);
  pf.recursive_roots.push_back(wprev.tree.back());
  tr.observe_bytes(wprev.tree.back().b, 32);
  for (int o = 0; o < ood(1); o++) {
    auto zpt = tr.sample_vec(n1);
    F128 y;
    Msg im = sc.introduce_eval(eq_table(zpt), y);
    tr.observe_f128(y);
    pf.ood_values.push_back(y);
    tr.observe_f128(im.u0);
    tr.observe_f128(im.u2);
    sc.glue(tr.sample());
  }
  pf.grinding_nonces.push_back(tr.grind(cfg.grinding_bits[0]));
  auto q0 = sample_queries(tr, block0, cfg.queries[0]);
  auto a0 = tr.sample_vec(ceil_log2(cfg.queries[0]));
  {
    pf.initial.proof = merkle_multi_proof(l0.tree, block0, q0);
    for (size_t p : q0) pf.initial.rows.emplace_back(l0.codeword.begin() + p * ni0, l0.codeword.begin() + (p + 1) * ni0);
  }
  {
    std::vector<F128> basis;
    F128 enf;
    induce(n1, pf.initial.rows, r_lane, q0, a0, basis, enf);
    Msg im = sc.introduce(std::move(basis));
    tr.observe_f128(im.u0);
    tr.observe_f128(im.u2);
    sc.glue(tr.sample());
    (void)enf;
  }
  for (int i = 0; i < cfg.steps; i++) {
    int ki = cfg.ks[i];
    std::vector<F128> level_rs;
    for (int j = 0; j < ki; j++) {
      uint32_t bits = fb(i + 1) > (uint32_t)j ? fb(i + 1) - j : 0;
      if (bits) pf.fold_nonces.push_back(tr.grind(bits));
      F128 r = tr.sample();
      Msg m = sc.fold(r);
      tr.observe_f128(m.u0);
      tr.observe_f128(m.u2);
      level_rs.push_back(r);
    }
    if (i == cfg.steps - 1) {
      pf.yr = sc.f;
      for (auto& v : pf.yr) tr.observe_f128(v);
      pf.grinding_nonces.push_back(tr.grind(cfg.grinding_bits[i + 1]));
      auto ql = sample_queries(tr, wprev.block_len, cfg.queries[i + 1]);
      pf.final_open = open_rows(wprev, ql);
      pf.sumcheck = sc.msgs;
      return pf;
    }
    int n_next = ceil_log2(sc.f.size());
    int lni = cfg.ks[i + 1];
    LigeroWitness wnext = ligero_commit(sc.f, n_next - lni, lni, cfg.log_inv_rates[i + 2]);
    pf.recursive_roots.push_back(wnext.tree.back());
    tr.observe_bytes(wnext.tree.back().b, 32);
    for (int o = 0; o < ood(i + 2); o++) {
      auto zpt = tr.sample_vec(n_next);
      F128 y;
      Msg im = sc.introduce_eval(eq_table(zpt), y);
      tr.observe_f128(y);
      pf.ood_values.push_back(y);
      tr.observe_f128(im.u0);
      tr.observe_f128(im.u2);
      sc.glue(tr.sample());
    }
    pf.grinding_nonces.push_back(tr.grind(cfg.grinding_bits[i + 1]));
    auto qi = sample_queries(tr, wprev.block_len, cfg.queries[i + 1]);
    auto ai = tr.sample_vec(ceil_log2(cfg.queries[i + 1]));
    LevelOpen lo = open_rows(wprev, qi);
    std::vector<F128> basis;
    F128 enf;
    induce(n_next, lo.rows, level_rs, qi, ai, basis, enf);
    pf.recursive.push_back(std::move(lo));
    Msg im = sc.introduce(std::move(basis));
    tr.observe_f128(im.u0);
    tr.observe_f128(im.u2);
    sc.glue(tr.sample());
    wprev = std::move(wnext);
  }
  return pf;
}

struct Quad {
  F128 c, b, a;
  static Quad from(F128 u0, F128 u2, F128 t) { return {u0, t + u2, u2}; }
  F128 eval(F128 r) const { return c + r * b + r * r * a; }
  static Quad fold(const Quad& p, const Quad& q, F128 al) { return {p.c + al * q.c, p.b + al * q.b, p.a + al * q.a}; }
};

static bool level_opens_ok(const Hash32& root, size_t block_len, const std::vector<size_t>& q, const LevelOpen& o,
                           size_t ni) {
  if (q.size() != o.rows.size()) return false;
  std::vector<Hash32> leaves;
  for (auto& row : o.rows) {
    if (row.size() != ni) return false;
    leaves.push_back(leaf_cv((const uint8_t*)row.data(), row.size() * 16));
  }
  return verify_merkle_multi_proof(root, block_len, q, leaves, o.proof);
}

static F128 enforced_sum(const LevelOpen& o, const std::vector<F128>& v, const std::vector<F128>& alpha) {
  auto eqv = eq_table(v);
  auto at = eq_table(alpha);
  F128 s;
  for (size_t i = 0; i < o.rows.size(); i++) s += at[i] * dot(o.rows[i].data(), eqv.data(), o.rows[i].size());
  return s;
}

// ligerito.rs:1879-1987: MLE of the induced basis at ris_for_basis ++ bits(y).
static std::vector<F128> induced_residual(int n, const std::vector<size_t>& q, const std::vector<F128>& alpha,
                                          const F128* ris, int prefix, int yr_log) {
  auto sks = sk_at_vk(n);
  auto at = eq_table(alpha);
  std::vector<F128> out((size_t)1 << yr_log);
  for (size_t i = 0; i < q.size(); i++) {
    auto w = what_at(n, sks, q[i]);
    F128 pre = one();
    for (int k = 0; k < prefix; k++) pre = pre * (one() + ris[k] * (one() + w[k]));
    for (size_t y = 0; y < out.size(); y++) {
      F128 suf = one();
      for (int j = 0; j < yr_log; j++)
        if ((y >> j) & 1) suf = suf * w[prefix + j];
      out[y] += at[i] * pre * suf;
    }
  }
  return out;
}

static bool ligerito_verify(const LigConfig& cfg, const LigeritoProof& pf, int log_n, F128 target,
                            const Hash32& root, const std::vector<F128>& b_dense, Transcript& tr, std::string* why) {
  auto fail = [&](const char* w) {
    if (why) *why = std::string("ligerito: ") + w;
    return false;
  };
  int k0 = cfg.initial_k, R = cfg.steps;
  if (!(pf.initial_root == root)) return fail("root");
  tr.label("flock-ligerito-basis-v0");
  tr.observe_f128(target);
  tr.observe_bytes(pf.initial_root.b, 32);
  size_t block0 = (size_t)1 << (log_n - k0 + cfg.log_inv_rates[0]);
  F128 t_r = target;
  size_t tx = 0;
  auto next_msg = [&](std::pair<F128, F128>& m) {
    if (tx >= pf.sumcheck.size()) return false;
    m = pf.sumcheck[tx++];
    tr.observe_f128(m.first);
    tr.observe_f128(m.second);
    return true;
  };
  std::pair<F128, F128> m;
  if (!next_msg(m)) return fail("transcript");
  Quad run = Quad::from(m.first, m.second, t_r);
  auto fb = [&](int lvl) { return (uint32_t)(lvl < (int)cfg.fold_bits.size() ? cfg.fold_bits[lvl] : 0); };
  auto ood = [&](int lvl) { return lvl < (int)cfg.ood.size() ? cfg.ood[lvl] : 0; };
  size_t fni = 0, oi = 0, ni = 0;
  struct OodCtx { std::vector<F128> z; size_t start; F128 beta; };
  struct LvlCtx { int n; std::vector<size_t> q; std::vector<F128> alpha; size_t start; F128 beta; };
  std::vector<OodCtx> oods;
  std::vector<LvlCtx> lvls;
  std::vector<F128> ris;
  for (int j = 0; j < k0; j++) {
    uint32_t bits = fb(0) > (uint32_t)j ? fb(0) - j : 0;
    if (bits) {
      if (fni >= pf.fold_nonces.size() || !tr.verify_pow(pf.fold_nonces[fni++], bits)) return fail("fold pow");
    }
    F128 r = tr.sample();
    ris.push_back(r);
    t_r = run.eval(r);
    if (!next_msg(m)) return fail("transcript");
    run = Quad::from(m.first, m.second, t_r);
  }
  if (pf.recursive_roots.empty()) return fail("roots");
  Hash32 prev_root = pf.recursive_roots[0];
  tr.observe_bytes(prev_root.b, 32);
  int n1 = log_n - k0;
  for (int o = 0; o < ood(1); o++) {
    auto z = tr.sample_vec(n1);
    if (oi >= pf.ood_values.size()) return fail("ood");
    F128 y = pf.ood_values[oi++];
    tr.observe_f128(y);
    if (!next_msg(m)) return fail("transcript");
    Quad iq = Quad::from(m.first, m.second, y);
    F128 beta = tr.sample();
    run = Quad::fold(run, iq, beta);
    t_r += beta * y;
    oods.push_back({z, (size_t)k0, beta});
  }
  if (ni >= pf.grinding_nonces.size() || !tr.verify_pow(pf.grinding_nonces[ni++], cfg.grinding_bits[0]))
    return fail("query pow 0");
  auto q0 = sample_queries(tr, block0, cfg.queries[0]);
  auto a0 = tr.sample_vec(ceil_log2(cfg.queries[0]));
  if (!level_opens_ok(pf.initial_root, block0, q0, pf.initial, (size_t)1 << k0)) return fail("L0 opens");
  F128 es0 = enforced_sum(pf.initial, ris, a0);
  if (!next_msg(m)) return fail("transcript");
  {
    Quad iq = Quad::from(m.first, m.second, es0);
    F128 beta = tr.sample();
    run = Quad::fold(run, iq, beta);
    t_r += beta * es0;
    lvls.push_back({n1, q0, a0, (size_t)k0, beta});
  }
  int prev_lni = cfg.ks[0];
  int prev_lmc = n1 - prev_lni;
  int prev_rate = cfg.log_inv_rates[1];
  size_t rp = 0;
  int n_cur = n1;
  for (int i = 0; i < R; i++) {
    int ki = cfg.ks[i];
    std::vector<F128> level_rs;
    for (int j = 0; j < ki; j++) {
      uint32_t bits = fb(i + 1) > (uint32_t)j ? fb(i + 1) - j : 0;
      if (bits) {
        if (fni >= pf.fold_nonces.size() || !tr.verify_pow(pf.fold_nonces[fni++], bits)) return fail("fold pow");
      }
      F128 r = tr.sample();
      ris.push_back(r);
      level_rs.push_back(r);
      t_r = run.eval(r);
      if (!next_msg(m)) return fail("transcript");
      run = Quad::from(m.first, m.second, t_r);
    }
    n_cur -= ki;
    if (i == R - 1) {
      if (tx != pf.sumcheck.size() || oi != pf.ood_values.size() || fni != pf.fold_nonces.size())
        return fail("trailing");
      if (pf.yr.size() != ((size_t)1 << n_cur)) return fail("yr size");
      for (auto& v : pf.yr) tr.observe_f128(v);
      if (ni >= pf.grinding_nonces.size() || !tr.verify_pow(pf.grinding_nonces[ni], cfg.grinding_bits[i + 1]))
        return fail("query pow last");
      size_t pbl = (size_t)1 << (prev_lmc + prev_rate);
      auto ql = sample_queries(tr, pbl, cfg.queries[i + 1]);
      auto al = tr.sample_vec(ceil_log2(cfg.queries[i + 1]));
      if (!level_opens_ok(prev_root, pbl, ql, pf.final_open, (size_t)1 << prev_lni)) return fail("last opens");
      F128 esl = enforced_sum(pf.final_open, level_rs, al);
      F128 bl = tr.sample();
      t_r += bl * esl;
      lvls.push_back({n_cur, ql, al, ris.size(), bl});
      int yl = n_cur;
      // dense basis residual: partial evaluation of b at ris (LSB first)
      std::vector<F128> bres = b_dense;
      for (F128 r : ris) fold_lsb(bres, r);
      if (bres.size() != pf.yr.size()) return fail("residual size");
      std::vector<std::vector<F128>> ind;
      for (auto& c : lvls) {
        int prefix = c.n - yl;
        ind.push_back(induced_residual(c.n, c.q, c.alpha, ris.data() + c.start, prefix, yl));
      }
      std::vector<std::vector<F128>> oodr;
      for (auto& c : oods) {
        int folded = (int)c.z.size() - yl;
        F128 sc = c.beta;
        for (int b2 = 0; b2 < folded; b2++) sc = sc * (one() + c.z[b2] + ris[c.start + b2]);
        std::vector<F128> tail(c.z.begin() + folded, c.z.end());
        auto t = eq_table(tail);
        for (auto& v : t) v = v * sc;
        oodr.push_back(t);
      }
      F128 inner;
      for (size_t y = 0; y < pf.yr.size(); y++) {
        F128 cy = bres[y];
        for (size_t k = 0; k < lvls.size(); k++) cy += lvls[k].beta * ind[k][y];
        for (auto& t : oodr) cy += t[y];
        inner += pf.yr[y] * cy;
      }
      if (inner != t_r) return fail("residual check");
      return true;
    }
    if ((size_t)(i + 1) >= pf.recursive_roots.size()) return fail("roots");
    Hash32 root_next = pf.recursive_roots[i + 1];
    tr.observe_bytes(root_next.b, 32);
    for (int o = 0; o < ood(i + 2); o++) {
      auto z = tr.sample_vec(n_cur);
      if (oi >= pf.ood_values.size()) return fail("ood");
      F128 y = pf.ood_values[oi++];
      tr.observe_f128(y);
      if (!next_msg(m)) return fail("transcript");
      Quad iq = Quad::from(m.first, m.second, y);
      F128 beta = tr.sample();
      run = Quad::fold(run, iq, beta);
      t_r += beta * y;
      oods.push_back({z, ris.size(), beta});
    }
    if (ni >= pf.grinding_nonces.size() || !tr.verify_pow(pf.grinding_nonces[ni++], cfg.grinding_bits[i + 1]))
      return fail("query pow");
    size_t pbl = (size_t)1 << (prev_lmc + prev_rate);
    auto qi = sample_queries(tr, pbl, cfg.queries[i + 1]);
    auto ai = tr.sample_vec(ceil_log2(cfg.queries[i + 1]));
    if (rp >= pf.recursive.size()) return fail("recursive proofs");
    const LevelOpen& lo = pf.recursive[rp++];
    if (!level_opens_ok(prev_root, pbl, qi, lo, (size_t)1 << prev_lni)) return fail("level opens");
    F128 esi = enforced_sum(lo, level_rs, ai);
    if (!next_msg(m)) return fail("transcript");
    Quad iq = Quad::from(m.first, m.second, esi);
    F128 beta = tr.sample();
    run = Quad::fold(run, iq, beta);
    t_r += beta * esi;
    lvls.push_back({n_cur, qi, ai, ris.size(), beta});
    prev_root = root_next;
    int kn = cfg.ks[i + 1];
    prev_lni = kn;
    prev_lmc = n_cur - kn;
    prev_rate = cfg.log_inv_rates[i + 2];
  }
  return fail("unreachable");
}

// ============================================================================
// Top level
// ============================================================================
static void bind_statement(Transcript& tr, const uint8_t digest[32], const Hash32& root) {
  tr.label("flock-r1cs-v0");
  tr.observe_bytes(digest, 32);
  tr.observe_bytes(root.b, 32);
}

struct RsOut {
  std::vector<F128> s_hat_v, eq_r;
  F128 claim;
};
static RsOut ring_switch_prove(const std::vector<F128>& z, const std::vector<F128>& x_full, Transcript& tr,
                               std::vector<F128>& rs_eq_ind) {
  RsOut o;
  tr.label("flock-ring-switch-v0");
  std::vector<F128> suffix(x_full.begin() + 1, x_full.end());
  auto t = eq_table(suffix);
  o.s_hat_v = fold_1b_rows(z, t);
  tr.observe_slice(o.s_hat_v.data(), 128);
  auto rpp = tr.sample_vec(7);
  o.eq_r = eq_table(rpp);
  auto u = transpose128(o.s_hat_v);
  o.claim = dot(u.data(), o.eq_r.data(), 128);
  rs_eq_ind = fold_b128(t, o.eq_r);
  return o;
}

// The R1CS proof (prover.rs:194-289); with `chain`, the hash-chain proof of
// chain_common.rs:290-346: after lincheck the packed-position fold and the
// shift sumcheck, then one opening over [ab, c] plus the packed-direct chain
// claim (pcs.rs:1055-1090).
static Bundle prove_impl(const std::vector<Compression>& blocks, int n_log, const uint8_t digest[32],
                         Transcript& tr, ChainBundle* chain, R1csClaimOut* claim_out) {
  Bundle out;
  Witness w = build_witness(blocks, n_log, true);
  int m = w.m;
  out.params.m = m;
  CommitData cd = commit(w.z, out.params);
  out.root = cd.root();
  bind_statement(tr, digest, out.root);
  ZcClaim zc;
  out.zc = zc_prove((const uint64_t*)w.a.data(), (const uint64_t*)w.b.data(), (const uint64_t*)w.z.data(), m, tr, zc);
  std::vector<F128> x_in(zc.mlv.begin(), zc.mlv.begin() + (K_LOG - K_SKIP));
  std::vector<F128> x_out(zc.mlv.begin() + (K_LOG - K_SKIP), zc.mlv.end());
  static SparseRows A, B;
  static bool have = false;
  if (!have) {
    build_matrices(A, B);
    have = true;
  }
  LcClaim lc;
  out.lc = lc_prove(w.stripe.data(), m, A, B, zc.z, x_in, x_out, tr, lc);
  std::vector<F128> pd_point;
  F128 pd_value;
  if (chain) {
    F128 tau = tr.sample_vec(1)[0];
    std::vector<F128> in_vals, out_vals;
    chain_fold_io(w.z, (size_t)1 << n_log, tau, in_vals, out_vals);
    ChainClaims cl;
    chain->shift = prove_chain_shift(in_vals, out_vals, tr, cl);
    pd_point = chain_claim_point(tau, cl);
    pd_value = cl.value;
  }
  if (claim_out) {  // R1csClaim { ab, c } (prover.rs:255-262; r1cs.rs:289-334, RowMajor)
    claim_out->ab_skip = lc.r_inner_skip;
    claim_out->ab_inner = lc.r_inner_rest;
    claim_out->ab_outer = x_out;
    claim_out->ab_value = lc.w;
    claim_out->c_skip = zc.z;
    claim_out->c_inner.assign(zc.r_rest.begin(), zc.r_rest.begin() + (K_LOG - K_SKIP));
    claim_out->c_outer.assign(zc.r_rest.begin() + (K_LOG - K_SKIP), zc.r_rest.end());
    claim_out->c_value = zc.c_eval;
  }
  // Claims [ab, c]; x_full = x_inner_rest ++ x_outer (prover.rs:138-146).
  std::vector<F128> x_ab(lc.r_inner_rest);
  x_ab.insert(x_ab.end(), x_out.begin(), x_out.end());
  const std::vector<F128>& x_c = zc.r_rest;
  tr.label("flock-pcs-open-batch-v0");
  std::vector<F128> rs0, rs1;
  RsOut o0 = ring_switch_prove(w.z, x_ab, tr, rs0);
  RsOut o1 = ring_switch_prove(w.z, x_c, tr, rs1);
  F128 g0 = tr.sample(), g1 = tr.sample();
  out.s_hat_v = {o0.s_hat_v, o1.s_hat_v};
  std::vector<F128> b(rs0.size());
  for (size_t i = 0; i < b.size(); i++) b[i] = g0 * rs0[i] + g1 * rs1[i];
  F128 target = g0 * o0.claim + g1 * o1.claim;
  if (chain) {
    tr.label("flock-pcs-packed-direct-v0");
    tr.observe_f128(pd_value);
    F128 g2 = tr.sample();
    auto e = eq_table(pd_point);
    for (size_t i = 0; i < b.size(); i++) b[i] += g2 * e[i];
    target += g2 * pd_value;
  }
  LigConfig cfg;
  if (!ligerito_config(m, 0, cfg)) throw std::runtime_error("no ligerito config for m");
  out.lig = ligerito_prove(cfg, w.z, std::move(b), target, cd, tr);
  return out;
}

Bundle prove(const std::vector<Compression>& blocks, int n_log, const uint8_t digest[32], const std::string& domain) {
  Transcript tr(domain);
  return prove_impl(blocks, n_log, digest, tr, nullptr, nullptr);
}

Bundle prove_with(const std::vector<Compression>& blocks, int n_log, const uint8_t digest[32], Transcript& tr,
                  R1csClaimOut* claim) {
  return prove_impl(blocks, n_log, digest, tr, nullptr, claim);
}

ChainBundle prove_chain(const std::vector<Compression>& blocks, int n_log, const uint8_t digest[32],
                        const std::string& domain) {
  if (blocks.empty() || blocks.size() != ((size_t)1 << n_log)) throw std::runtime_error("chain: steps must fill 2^n");
  ChainBundle cb;
  Transcript tr(domain);
  cb.b = prove_impl(blocks, n_log, digest, tr, &cb, nullptr);
  uint32_t o[16];
  const Compression& l = blocks.back();
  b3_compress(l.cv, l.m, l.counter, l.block_len, l.flags, o);
  cb.cv0_phys = cv_to_phys(blocks[0].cv);
  cb.cvlast_phys = cv_to_phys(o);
  return cb;
}

static bool verify_impl(const Bundle& bd, int m, const uint8_t digest[32], const SparseRows& A, const SparseRows& B,
                        Transcript& tr, std::string* why, const ChainBundle* chain) {
  if (bd.params.m != m || bd.params.log_inv_rate != 1 || bd.params.log_batch_size != 6) {
    if (why) *why = "params";
    return false;
  }
  bind_statement(tr, digest, bd.root);
  ZcClaim zc;
  if (!zc_verify(bd.zc, m, tr, zc, why)) return false;
  std::vector<F128> x_in(zc.mlv.begin(), zc.mlv.begin() + (K_LOG - K_SKIP));
  std::vector<F128> x_out(zc.mlv.begin() + (K_LOG - K_SKIP), zc.mlv.end());
  LcClaim lc;
  if (!lc_verify(bd.lc, A, B, zc.z, x_in, zc.a_eval, zc.b_eval, tr, lc, why)) return false;
  std::vector<F128> pd_point;
  F128 pd_value;
  if (chain) {
    if (chain->cv0_phys.size() > 256 || chain->cvlast_phys.size() > 256) {
      if (why) *why = "chain endpoints";
      return false;
    }
    F128 tau = tr.sample_vec(1)[0];
    F128 x0 = fold_public_phys(chain->cv0_phys, tau), xl = fold_public_phys(chain->cvlast_phys, tau);
    ChainClaims cl;
    if (!verify_chain_shift(chain->shift, x0, xl, m - K_LOG, tr, cl)) {
      if (why) *why = "chain shift";
      return false;
    }
    pd_point = chain_claim_point(tau, cl);
    pd_value = cl.value;
  }
  std::vector<F128> x_ab(lc.r_inner_rest);
  x_ab.insert(x_ab.end(), x_out.begin(), x_out.end());
  const std::vector<F128>& x_c = zc.r_rest;
  if (bd.s_hat_v.size() != 2) {
    if (why) *why = "ring switch count";
    return false;
  }
  tr.label("flock-pcs-open-batch-v0");
  const std::vector<F128>* xs[2] = {&x_ab, &x_c};
  F128 zsk[2] = {lc.r_inner_skip, zc.z}, val[2] = {lc.w, zc.c_eval}, claims[2];
  std::vector<F128> eqr[2];
  for (int k = 0; k < 2; k++) {
    if (bd.s_hat_v[k].size() != 128) {
      if (why) *why = "s_hat_v size";
      return false;
    }
    tr.label("flock-ring-switch-v0");
    tr.observe_slice(bd.s_hat_v[k].data(), 128);
    auto w = claim_weights(zsk[k], (*xs[k])[0]);
    if (dot(w.data(), bd.s_hat_v[k].data(), 128) != val[k]) {
      if (why) *why = "ring switch claim";
      return false;
    }
    auto rpp = tr.sample_vec(7);
    eqr[k] = eq_table(rpp);
    auto u = transpose128(bd.s_hat_v[k]);
    claims[k] = dot(u.data(), eqr[k].data(), 128);
  }
  F128 g0 = tr.sample(), g1 = tr.sample();
  F128 target = g0 * claims[0] + g1 * claims[1];
  std::vector<F128> b;
  {
    std::vector<F128> s0(x_ab.begin() + 1, x_ab.end()), s1(x_c.begin() + 1, x_c.end());
    auto r0 = fold_b128(eq_table(s0), eqr[0]);
    auto r1 = fold_b128(eq_table(s1), eqr[1]);
    b.resize(r0.size());
    for (size_t i = 0; i < b.size(); i++) b[i] = g0 * r0[i] + g1 * r1[i];
  }
  if (chain) {
    tr.label("flock-pcs-packed-direct-v0");
    tr.observe_f128(pd_value);
    F128 g2 = tr.sample();
    auto e = eq_table(pd_point);
    for (size_t i = 0; i < b.size(); i++) b[i] += g2 * e[i];
    target += g2 * pd_value;
  }
  LigConfig cfg;
  if (!ligerito_config(m, 0, cfg)) return false;
  return ligerito_verify(cfg, bd.lig, m - 7, target, bd.root, b, tr, why);
}

bool verify(const Bundle& bd, int m, const uint8_t digest[32], const SparseRows& A, const SparseRows& B,
            const std::string& domain, std::string* why) {
  Transcript tr(domain);
  return verify_impl(bd, m, digest, A, B, tr, why, nullptr);
}

bool verify_with(const Bundle& bd, int m, const uint8_t digest[32], const SparseRows& A, const SparseRows& B,
                 Transcript& tr, std::string* why) {
  return verify_impl(bd, m, digest, A, B, tr, why, nullptr);
}

bool verify_chain(const ChainBundle& cb, int m, const uint8_t digest[32], const SparseRows& A, const SparseRows& B,
                  const std::string& domain, std::string* why) {
  Transcript tr(domain);
  return verify_impl(cb.b, m, digest, A, B, tr, why, &cb);
}

// ============================================================================
// Wire format: "FLOCK" 0x04 0x02 + bincode-fixint (proof_io.rs:161-208)
// ============================================================================
struct W {
  std::vector<uint8_t> v;
  void u8(uint8_t x) { v.push_back(x); }
  void u32(uint32_t x) { for (int i = 0; i < 4; i++) v.push_back((uint8_t)(x >> (8 * i))); }
  void u64(uint64_t x) { for (int i = 0; i < 8; i++) v.push_back((uint8_t)(x >> (8 * i))); }
  void f(F128 x) { u64(x.lo); u64(x.hi); }
  void h(const Hash32& x) { v.insert(v.end(), x.b, x.b + 32); }
  void fv(const std::vector<F128>& x) { u64(x.size()); for (auto& e : x) f(e); }
  void pv(const std::vector<std::pair<F128, F128>>& x) { u64(x.size()); for (auto& e : x) { f(e.first); f(e.second); } }
  void hv(const std::vector<Hash32>& x) { u64(x.size()); for (auto& e : x) h(e); }
  void uv(const std::vector<uint64_t>& x) { u64(x.size()); for (auto e : x) u64(e); }
  void open(const LevelOpen& o) { u64(o.rows.size()); for (auto& r : o.rows) fv(r); hv(o.proof); }
};

// Commitment, zerocheck, lincheck, [chain shift,] BatchOpeningProofLigerito.
static void write_body(W& w, const Bundle& b, const ChainShiftProof* shift) {
  // Commitment { root, params { m, log_inv_rate, log_batch_size, profile, merkle_hash } }
  w.h(b.root);
  w.u64(b.params.m);
  w.u64(b.params.log_inv_rate);
  w.u64(b.params.log_batch_size);
  w.u32(b.params.profile);
  w.u32(b.params.merkle_hash);
  // ZerocheckProof
  w.fv(b.zc.round1_ab);
  w.fv(b.zc.round1_c);
  w.pv(b.zc.rounds);
  w.f(b.zc.final_a);
  w.f(b.zc.final_b);
  w.f(b.zc.final_c);
  // LincheckProof
  w.pv(b.lc.rounds);
  w.fv(b.lc.z_partial);
  // ChainShiftProof { rounds, g_at_point } (chain.rs:105-116)
  if (shift) {
    w.pv(shift->rounds);
    w.f(shift->g_at_point);
  }
  // BatchOpeningProofLigerito
  w.u64(b.s_hat_v.size());
  for (auto& s : b.s_hat_v) w.fv(s);
  const LigeritoProof& l = b.lig;
  w.h(l.initial_root);
  w.open(l.initial);
  w.hv(l.recursive_roots);
  w.u64(l.recursive.size());
  for (auto& o : l.recursive) w.open(o);
  w.fv(l.yr);
  w.open(l.final_open);
  w.pv(l.sumcheck);
  w.uv(l.grinding_nonces);
  w.fv(l.ood_values);
  w.uv(l.fold_nonces);
}

static void write_header(W& w, uint8_t flavor) {
  const char* magic = "FLOCK";
  for (int i = 0; i < 5; i++) w.u8((uint8_t)magic[i]);
  w.u8(4);
  w.u8(flavor);
}

std::vector<uint8_t> encode_bundle(const Bundle& b) {
  W w;
  write_header(w, 2);
  write_body(w, b, nullptr);
  return w.v;
}

// proof_io.rs:486-493: flavor 3, HashKind::Blake3 = 0, the body with the
// shift proof, then the endpoint bits as Vec<bool> (one byte each).
std::vector<uint8_t> encode_chain_bundle(const ChainBundle& cb) {
  W w;
  write_header(w, 3);
  w.u32(0);
  write_body(w, cb.b, &cb.shift);
  for (const auto* v : {&cb.cv0_phys, &cb.cvlast_phys}) {
    w.u64(v->size());
    for (uint8_t x : *v) w.u8(x);
  }
  return w.v;
}

struct R {
  const uint8_t* p;
  size_t n, at = 0;
  bool ok = true;
  bool need(size_t k) { if (at + k > n) ok = false; return ok; }
  uint8_t u8() { if (!need(1)) return 0; return p[at++]; }
  uint32_t u32() { if (!need(4)) return 0; uint32_t x = 0; for (int i = 0; i < 4; i++) x |= (uint32_t)p[at + i] << (8 * i); at += 4; return x; }
  uint64_t u64() { if (!need(8)) return 0; uint64_t x = 0; for (int i = 0; i < 8; i++) x |= (uint64_t)p[at + i] << (8 * i); at += 8; return x; }
  F128 f() { F128 x; x.lo = u64(); x.hi = u64(); return x; }
  Hash32 h() { Hash32 x; memset(x.b, 0, 32); if (need(32)) { memcpy(x.b, p + at, 32); at += 32; } return x; }
  size_t len(size_t elem) { uint64_t k = u64(); if (!ok || k > (n - at) / (elem ? elem : 1)) { ok = false; return 0; } return (size_t)k; }
  std::vector<F128> fv() { size_t k = len(16); std::vector<F128> v(k); for (auto& e : v) e = f(); return v; }
  std::vector<std::pair<F128, F128>> pv() { size_t k = len(32); std::vector<std::pair<F128, F128>> v(k); for (auto& e : v) { e.first = f(); e.second = f(); } return v; }
  std::vector<Hash32> hv() { size_t k = len(32); std::vector<Hash32> v(k); for (auto& e : v) e = h(); return v; }
  std::vector<uint64_t> uv() { size_t k = len(8); std::vector<uint64_t> v(k); for (auto& e : v) e = u64(); return v; }
  LevelOpen open() { LevelOpen o; size_t k = len(8); o.rows.resize(k); for (auto& r : o.rows) r = fv(); o.proof = hv(); return o; }
};

static void read_body(R& r, Bundle& b, ChainShiftProof* shift) {
  b.root = r.h();
  b.params.m = (int)r.u64();
  b.params.log_inv_rate = (int)r.u64();
  b.params.log_batch_size = (int)r.u64();
  b.params.profile = (int)r.u32();
  b.params.merkle_hash = (int)r.u32();
  b.zc.round1_ab = r.fv();
  b.zc.round1_c = r.fv();
  b.zc.rounds = r.pv();
  b.zc.final_a = r.f();
  b.zc.final_b = r.f();
  b.zc.final_c = r.f();
  b.lc.rounds = r.pv();
  b.lc.z_partial = r.fv();
  if (shift) {
    shift->rounds = r.pv();
    shift->g_at_point = r.f();
  }
  size_t k = r.len(8);
  b.s_hat_v.resize(k);
  for (auto& s : b.s_hat_v) s = r.fv();
  LigeritoProof& l = b.lig;
  l.initial_root = r.h();
  l.initial = r.open();
  l.recursive_roots = r.hv();
  size_t nr = r.len(8);
  l.recursive.resize(nr);
  for (auto& o : l.recursive) o = r.open();
  l.yr = r.fv();
  l.final_open = r.open();
  l.sumcheck = r.pv();
  l.grinding_nonces = r.uv();
  l.ood_values = r.fv();
  l.fold_nonces = r.uv();
}

bool decode_bundle(const uint8_t* p, size_t n, Bundle& b) {
  if (n < 7 || memcmp(p, "FLOCK", 5) != 0 || p[5] != 4 || p[6] != 2) return false;
  R r{p, n, 7};
  read_body(r, b, nullptr);
  return r.ok && r.at == n;  // trailing bytes rejected
}

bool decode_chain_bundle(const uint8_t* p, size_t n, ChainBundle& cb) {
  if (n < 7 || memcmp(p, "FLOCK", 5) != 0 || p[5] != 4 || p[6] != 3) return false;
  R r{p, n, 7};
  if (r.u32() != 0) return false;  // HashKind::Blake3 only
  read_body(r, cb.b, &cb.shift);
  for (auto* v : {&cb.cv0_phys, &cb.cvlast_phys}) {
    size_t k = r.len(1);
    v->resize(k);
    for (auto& x : *v) {
      x = r.u8();
      if (x > 1) return false;  // bincode bools are 0 or 1
    }
  }
  return r.ok && r.at == n;
}

}  // namespace oracle

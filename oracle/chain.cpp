// Oracle restatement of the BLAKE3 hash-chain relation (test infrastructure only).
//
// The chain statement glues 2^n committed compressions into a sequential
// chain cv_{i+1} = out_lo(compress_i) with public endpoints. It follows
// crates/flock-prover/src/chain.rs (shift MLE :78-100, shift sumcheck prover
// :155-233, verifier :238-302), the region fold and claim point of
// crates/flock-prover/src/r1cs_hashes/chain_common.rs (:88-113 public fold,
// :124-176 fold_in_out, :196-231 claim point) with BLAKE3's layout
// (r1cs_hashes/blake3.rs:3750-3770: cv in bits [0, 256), out_lo in
// [256, 512) of each 2^14-bit block), and the flock_chain CLI's honest-chain
// builder (crates/flock-prover/src/bin/flock_chain.rs:222-262).
#include <cstring>

#include "protocol.h"

namespace oracle {

static inline F128 one() { return f128(1); }

// chain.rs:78-100: sum_j [prod_{l<j} a_l (1 + b_l)] (1 + a_j) b_j [prod_{l>j} (1 + a_l + b_l)].
F128 shift_mle(const std::vector<F128>& a, const std::vector<F128>& b) {
  const size_t n = a.size();
  std::vector<F128> pre(n + 1, one()), suf(n + 1, one());
  for (size_t j = 0; j < n; j++) pre[j + 1] = pre[j] * (a[j] * (one() + b[j]));
  for (size_t j = n; j-- > 0;) suf[j] = suf[j + 1] * (one() + a[j] + b[j]);
  F128 acc;
  for (size_t j = 0; j < n; j++) acc += pre[j] * ((one() + a[j]) * b[j]) * suf[j + 1];
  return acc;
}

static F128 eq_eval(const std::vector<F128>& a, const std::vector<F128>& b) {
  F128 acc = one();
  for (size_t j = 0; j < a.size(); j++) acc = acc * (one() + a[j] + b[j]);
  return acc;
}

// chain.rs:155-233. Tables over (y, s0) with s0 the high bit: W(y, 0) =
// eq(tau, y - 1) + alpha [y == 0], W(y, 1) = eq(tau, y); g = [In || Out].
// Each round sends (q(1), q(inf)) and binds the top remaining variable.
ChainShiftProof prove_chain_shift(const std::vector<F128>& in_vals, const std::vector<F128>& out_vals, Transcript& tr,
                                  ChainClaims& cl) {
  const size_t N = in_vals.size();
  int n = 0;
  while (((size_t)1 << n) < N) n++;
  auto tau = tr.sample_vec(n);
  F128 alpha = tr.sample();
  auto eqt = eq_table(tau);
  std::vector<F128> wt(2 * N), g(2 * N);
  for (size_t y = 1; y < N; y++) wt[y] = eqt[y - 1];
  wt[0] += alpha;
  for (size_t y = 0; y < N; y++) wt[N + y] = eqt[y];
  for (size_t y = 0; y < N; y++) {
    g[y] = in_vals[y];
    g[N + y] = out_vals[y];
  }
  ChainShiftProof pf;
  const int d = n + 1;
  std::vector<F128> rs;
  for (int k = 0; k < d; k++) {
    size_t h = g.size() / 2;
    F128 e1, ei;
    for (size_t i = 0; i < h; i++) {
      e1 += wt[i + h] * g[i + h];
      ei += (wt[i + h] + wt[i]) * (g[i + h] + g[i]);
    }
    tr.observe_f128(e1);
    tr.observe_f128(ei);
    F128 r = tr.sample();
    for (size_t i = 0; i < h; i++) {
      wt[i] = wt[i] + r * (wt[i + h] + wt[i]);
      g[i] = g[i] + r * (g[i + h] + g[i]);
    }
    wt.resize(h);
    g.resize(h);
    pf.rounds.push_back({e1, ei});
    rs.push_back(r);
  }
  std::vector<F128> full(d);
  for (int k = 0; k < d; k++) full[d - 1 - k] = rs[k];
  cl.instance_point.assign(full.begin(), full.begin() + n);
  cl.sel0 = full[n];
  cl.value = g[0];
  pf.g_at_point = g[0];
  return pf;
}

// chain.rs:238-302.
bool verify_chain_shift(const ChainShiftProof& pf, F128 x0, F128 xlast, int n, Transcript& tr, ChainClaims& cl) {
  const int d = n + 1;
  if ((int)pf.rounds.size() != d) return false;
  auto tau = tr.sample_vec(n);
  F128 alpha = tr.sample();
  F128 ones = one();
  for (auto& t : tau) ones = ones * t;
  F128 claim = ones * xlast + alpha * x0;
  std::vector<F128> rs;
  for (auto& m : pf.rounds) {
    tr.observe_f128(m.first);
    tr.observe_f128(m.second);
    F128 r = tr.sample();
    F128 e0 = claim + m.first;
    F128 c1 = e0 + m.first + m.second;
    claim = m.second * r * r + c1 * r + e0;
    rs.push_back(r);
  }
  std::vector<F128> full(d);
  for (int k = 0; k < d; k++) full[d - 1 - k] = rs[k];
  std::vector<F128> tp(full.begin(), full.begin() + n);
  F128 s0 = full[n];
  F128 eq_t0 = one();
  for (auto& t : tp) eq_t0 = eq_t0 * (one() + t);
  F128 w = shift_mle(tau, tp) * (one() + s0) + eq_eval(tau, tp) * s0 + alpha * eq_t0 * (one() + s0);
  if (claim != w * pf.g_at_point) return false;
  cl.instance_point = tp;
  cl.sel0 = s0;
  cl.value = pf.g_at_point;
  return true;
}

// chain_common.rs:124-176 for BLAKE3 (row-major words, 128 packed words per
// block, tau_pos of length 1): in[i] = eq(tau, 0) z[128 i] + eq(tau, 1) z[128 i + 1],
// out[i] the same at words 128 i + 2, 128 i + 3.
void chain_fold_io(const std::vector<F128>& z, size_t n_inst, F128 tau, std::vector<F128>& in_vals,
                   std::vector<F128>& out_vals) {
  F128 e0 = one() + tau, e1 = tau;
  in_vals.resize(n_inst);
  out_vals.resize(n_inst);
  for (size_t i = 0; i < n_inst; i++) {
    const F128* w = &z[i * (K / 128)];
    in_vals[i] = e0 * w[0] + e1 * w[1];
    out_vals[i] = e0 * w[2] + e1 * w[3];
  }
}

// chain_common.rs:196-231 (row-major): [tau_pos, sel0, 0^5, instance...].
std::vector<F128> chain_claim_point(F128 tau, const ChainClaims& cl) {
  std::vector<F128> p;
  p.push_back(tau);
  p.push_back(cl.sel0);
  for (int i = 0; i < K_LOG - 8 - 1; i++) p.push_back(F128());
  p.insert(p.end(), cl.instance_point.begin(), cl.instance_point.end());
  return p;
}

// chain_common.rs:88-113: pack the 256 region bits into two F128 (bit b of
// word pos = phys[128 pos + b]) and take the eq(tau)-weighted sum.
F128 fold_public_phys(const std::vector<uint8_t>& phys, F128 tau) {
  F128 w[2];
  for (size_t i = 0; i < phys.size() && i < 256; i++) {
    if (!phys[i]) continue;
    size_t pos = i / 128, b = i % 128;
    if (b < 64) w[pos].lo |= 1ULL << b;
    else w[pos].hi |= 1ULL << (b - 64);
  }
  return (one() + tau) * w[0] + tau * w[1];
}

// blake3.rs:3762-3770: physical bit 32 w + b = bit b of word w.
std::vector<uint8_t> cv_to_phys(const uint32_t cv[8]) {
  std::vector<uint8_t> p(256);
  for (int w = 0; w < 8; w++)
    for (int b = 0; b < 32; b++) p[32 * w + b] = (uint8_t)((cv[w] >> b) & 1);
  return p;
}

// bin/flock_chain.rs:180-196, :222-245: SplitMix64 words (low 32 bits of each
// draw), 16 per message block; counter 0, block_len 64, flags 0; each cv is the
// previous compression's out_lo.
std::vector<Compression> chain_inputs(size_t steps, uint64_t seed, const uint32_t cv0[8]) {
  uint64_t s = seed;
  auto nx = [&]() {
    s += 0x9E3779B97F4A7C15ULL;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  };
  std::vector<Compression> v(steps);
  uint32_t cv[8];
  memcpy(cv, cv0 ? cv0 : B3_IV, 32);
  for (size_t i = 0; i < steps; i++) {
    Compression& c = v[i];
    memcpy(c.cv, cv, 32);
    for (int j = 0; j < 16; j++) c.m[j] = (uint32_t)nx();
    c.counter = 0;
    c.block_len = 64;
    c.flags = 0;
    uint32_t out[16];
    b3_compress(c.cv, c.m, 0, 64, 0, out);
    memcpy(cv, out, 32);
  }
  return v;
}

}  // namespace oracle

// C entry points of the oracle library for the test harness (ctypes).
// Test infrastructure only.
#include <cstdio>
#include <cstring>

#include "oracle.h"

using namespace oracle;

extern "C" {

void oracle_gf_mul(const uint64_t* a, const uint64_t* b, uint64_t* out) {
  F128 r = gf_mul(f128(a[0], a[1]), f128(b[0], b[1]));
  out[0] = r.lo;
  out[1] = r.hi;
}
// Products of count pseudo-random operand pairs (SplitMix64 from seed) by
// gf_mul and by the portable code; returns how many differ.
size_t oracle_gf_crosscheck(size_t count, uint64_t seed) {
  uint64_t s = seed;
  auto next = [&s]() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  size_t bad = 0;
  for (size_t i = 0; i < count; i++) {
    F128 a = f128(next(), next()), b = f128(next(), next());
    if (i % 7 == 0) a.hi = 0;         // sparse operands too
    if (i % 11 == 0) b.lo = ~0ull;
    if (gf_mul(a, b) != gf_mul_portable(a, b)) bad++;
  }
  return bad;
}
int oracle_gf_uses_pmull() { return gf_mul_uses_pmull(); }
void oracle_gf_mul_portable(const uint64_t* a, const uint64_t* b, uint64_t* out) {
  F128 r = gf_mul_portable(f128(a[0], a[1]), f128(b[0], b[1]));
  out[0] = r.lo;
  out[1] = r.hi;
}
void oracle_gf_inv(const uint64_t* a, uint64_t* out) {
  F128 r = gf_inv(f128(a[0], a[1]));
  out[0] = r.lo;
  out[1] = r.hi;
}
void oracle_phi8(uint8_t v, uint64_t* out) {
  F128 r = phi8(v);
  out[0] = r.lo;
  out[1] = r.hi;
}
uint8_t oracle_gf8_mul(uint8_t a, uint8_t b) { return gf8_mul(a, b); }

void oracle_b3_compress(const uint32_t* cv, const uint32_t* block, uint64_t counter, uint32_t block_len,
                        uint32_t flags, uint32_t* out16) {
  b3_compress(cv, block, counter, block_len, flags, out16);
}
void oracle_b3_hash(const uint8_t* data, size_t len, uint8_t* out32) { b3_hash(data, len, out32); }
void oracle_b3_xof(const uint8_t* data, size_t len, uint8_t* out, size_t out_len) {
  Blake3 h;
  h.update(data, len);
  h.finalize_xof(out, out_len);
}
// Parent chaining values of n node pairs: out[i] = parent(children[2i], children[2i+1]).
void oracle_parent_cvs(const uint8_t* children, size_t n, uint8_t* out) {
  for (size_t i = 0; i < n; i++) b3_parent_cv(children + 64 * i, children + 64 * i + 32, out + 32 * i);
}
void oracle_leaf_cv(const uint8_t* data, size_t len, uint8_t* out32) {
  Hash32 h = leaf_cv(data, len);
  memcpy(out32, h.b, 32);
}

// Compression records are 8+16 u32, u64 counter, u32 block_len, u32 flags
// (112 bytes, matching the C-ABI flock_compression layout).
void oracle_generate_compressions(uint32_t log2_size, uint64_t seed, int canary, Compression* out) {
  auto v = canary ? canary_compressions(log2_size) : generate_compressions(log2_size, seed);
  memcpy(out, v.data(), v.size() * sizeof(Compression));
}
size_t oracle_compression_size() { return sizeof(Compression); }

// z/a/b: 2^(m-7) * 16 bytes each; stripe: 2^m / 8 bytes (may be null).
void oracle_witness(const Compression* blocks, size_t n, int n_blocks_log, uint64_t* z, uint64_t* a,
                    uint64_t* b, uint8_t* stripe) {
  std::vector<Compression> v(blocks, blocks + n);
  Witness w = build_witness(v, n_blocks_log, stripe != nullptr);
  size_t bytes = w.z.size() * 16;
  memcpy(z, w.z.data(), bytes);
  if (a) memcpy(a, w.a.data(), bytes);
  if (b) memcpy(b, w.b.data(), bytes);
  if (stripe) memcpy(stripe, w.stripe.data(), w.stripe.size());
}

void oracle_statement_digest(int m, uint8_t* out32) {
  SparseRows A, B;
  build_matrices(A, B);
  statement_digest(m, A, B, out32);
}

// Returns the total nonzero count; fills per-row lengths (K entries each) and,
// when cols != null, the concatenated column indices of A then B.
size_t oracle_matrices(uint32_t* a_len, uint32_t* b_len, uint32_t* cols) {
  SparseRows A, B;
  build_matrices(A, B);
  size_t nnz = 0, at = 0;
  for (int i = 0; i < K; i++) {
    if (a_len) a_len[i] = (uint32_t)A.rows[i].size();
    nnz += A.rows[i].size();
  }
  for (int i = 0; i < K; i++) {
    if (b_len) b_len[i] = (uint32_t)B.rows[i].size();
    nnz += B.rows[i].size();
  }
  if (cols) {
    for (int i = 0; i < K; i++)
      for (uint32_t c : A.rows[i]) cols[at++] = c;
    for (int i = 0; i < K; i++)
      for (uint32_t c : B.rows[i]) cols[at++] = c;
  }
  return nnz;
}

void oracle_ntt_twiddles(int dim, uint64_t* out) {
  NttF128 ntt(dim);
  memcpy(out, ntt.twiddles.data(), ntt.twiddles.size() * 16);
}

void oracle_ntt_interleaved(uint64_t* data, size_t n_total, size_t num_ntts, int start_layer) {
  size_t n = n_total / num_ntts;
  int ld = 0;
  while (((size_t)1 << ld) < n) ld++;
  NttF128 ntt(ld);
  ntt.forward_interleaved((F128*)data, n_total, num_ntts, start_layer);
}

// Flat Merkle tree of n_leaves equal leaves over data (2*n_leaves-1 nodes).
void oracle_merkle_tree(const uint8_t* data, size_t len, size_t n_leaves, uint8_t* tree_out) {
  auto t = merkle_tree(data, len, n_leaves);
  memcpy(tree_out, t.data(), t.size() * 32);
}

// PCS commit of a packed witness z (2^(m-7) F128). Writes the 32-byte root,
// and the codeword / flat tree when the pointers are non-null.
void oracle_commit(const uint64_t* z, int m, int log_inv_rate, int log_batch_size, uint8_t* root,
                   uint64_t* codeword_out, uint8_t* tree_out) {
  PcsParams p;
  p.m = m;
  p.log_inv_rate = log_inv_rate;
  p.log_batch_size = log_batch_size;
  std::vector<F128> zv((const F128*)z, (const F128*)z + ((size_t)1 << (m - 7)));
  CommitData c = commit(zv, p);
  memcpy(root, c.root().b, 32);
  if (codeword_out) memcpy(codeword_out, c.codeword.data(), c.codeword.size() * 16);
  if (tree_out) memcpy(tree_out, c.tree.data(), c.tree.size() * 32);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Protocol entry points.
// ---------------------------------------------------------------------------
#include "protocol.h"

#include <map>
#include <mutex>

namespace {
struct Mats {
  SparseRows A, B;
  Mats() { build_matrices(A, B); }
};
const Mats& mats() {
  static const Mats m;
  return m;
}
// Statement digest per m, cached (setup-time work in the reference too).
void digest_for(int m, uint8_t out[32]) {
  static std::mutex mu;
  static std::map<int, std::array<uint8_t, 32>> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(m);
  if (it == cache.end()) {
    std::array<uint8_t, 32> d;
    statement_digest(m, mats().A, mats().B, d.data());
    it = cache.emplace(m, d).first;
  }
  memcpy(out, it->second.data(), 32);
}
}  // namespace

extern "C" {

// Builds and caches the base matrices and the statement digest of m (the
// setup every proof of that m reuses), so a timed proof excludes them.
void oracle_warm(int m) {
  uint8_t dg[32];
  digest_for(m, dg);
}

// Proves n compressions (padded to 2^n_blocks_log slots); writes the wire bytes.
// Returns 0, or -5 when cap is too small (len receives the needed size).
int oracle_prove(const Compression* blocks, size_t n, int n_blocks_log, uint8_t* out, size_t cap, size_t* len) {
  std::vector<Compression> v(blocks, blocks + n);
  uint8_t dg[32];
  digest_for(K_LOG + n_blocks_log, dg);
  Bundle b = prove(v, n_blocks_log, dg);
  auto bytes = encode_bundle(b);
  *len = bytes.size();
  if (bytes.size() > cap) return -5;
  memcpy(out, bytes.data(), bytes.size());
  return 0;
}

// Caller-owned transcripts (the Challenger seam of prove_fast): the oracle's
// FsChallenger restatement behind an opaque pointer.
void* oracle_transcript_new(const uint8_t* domain, size_t n) {
  return new Transcript(std::string((const char*)domain, n));
}
void* oracle_transcript_clone(const void* t) { return new Transcript(*(const Transcript*)t); }
void oracle_transcript_free(void* t) { delete (Transcript*)t; }
void oracle_transcript_label(void* t, const uint8_t* p, size_t n) {
  ((Transcript*)t)->label(std::string((const char*)p, n));
}
void oracle_transcript_observe_f128(void* t, const uint64_t* v) { ((Transcript*)t)->observe_f128(f128(v[0], v[1])); }
void oracle_transcript_observe_slice(void* t, const uint64_t* v, size_t n) {
  ((Transcript*)t)->observe_slice((const F128*)v, n);
}
void oracle_transcript_observe_bytes(void* t, const uint8_t* p, size_t n) { ((Transcript*)t)->observe_bytes(p, n); }
void oracle_transcript_sample(void* t, uint64_t* out) {
  F128 v = ((Transcript*)t)->sample();
  out[0] = v.lo;
  out[1] = v.hi;
}
void oracle_transcript_sample_vec(void* t, size_t n, uint64_t* out) {
  auto v = ((Transcript*)t)->sample_vec(n);
  memcpy(out, v.data(), n * 16);
}

// oracle_prove with the caller's transcript, which the proof advances.
// claim (F128 entries, may be null): ab z_skip, ab value, c z_skip, c value,
// then ab x_inner_rest (8), ab x_outer (m - 14), c x_inner_rest (8), c x_outer.
int oracle_prove_tr(const Compression* blocks, size_t n, int n_blocks_log, void* t, uint8_t* out, size_t cap,
                    size_t* len, uint64_t* claim) {
  std::vector<Compression> v(blocks, blocks + n);
  uint8_t dg[32];
  digest_for(K_LOG + n_blocks_log, dg);
  R1csClaimOut c;
  Bundle b = prove_with(v, n_blocks_log, dg, *(Transcript*)t, &c);
  auto bytes = encode_bundle(b);
  *len = bytes.size();
  if (claim) {
    std::vector<F128> flat = {c.ab_skip, c.ab_value, c.c_skip, c.c_value};
    for (auto* part : {&c.ab_inner, &c.ab_outer, &c.c_inner, &c.c_outer}) flat.insert(flat.end(), part->begin(), part->end());
    memcpy(claim, flat.data(), flat.size() * 16);
  }
  if (bytes.size() > cap) return -5;
  memcpy(out, bytes.data(), bytes.size());
  return 0;
}

// oracle_verify with the caller's transcript (advanced by the replay).
int oracle_verify_tr(const uint8_t* bytes, size_t len, int m, void* t, char* why, size_t why_cap) {
  Bundle b;
  if (!decode_bundle(bytes, len, b)) {
    if (why && why_cap) snprintf(why, why_cap, "malformed");
    return -1;
  }
  uint8_t dg[32];
  digest_for(m, dg);
  std::string w;
  bool ok = verify_with(b, m, dg, mats().A, mats().B, *(Transcript*)t, &w);
  if (why && why_cap) snprintf(why, why_cap, "%s", ok ? "ok" : w.c_str());
  return ok ? 0 : -2;
}

// 0 = accepted; -1 = malformed bytes; -2 = rejected. why (may be null) gets a
// short reason.
int oracle_verify(const uint8_t* bytes, size_t len, int m, char* why, size_t why_cap) {
  Bundle b;
  if (!decode_bundle(bytes, len, b)) {
    if (why && why_cap) snprintf(why, why_cap, "malformed");
    return -1;
  }
  uint8_t dg[32];
  digest_for(m, dg);
  std::string w;
  bool ok = verify(b, m, dg, mats().A, mats().B, "flock-bench-v0", &w);
  if (why && why_cap) snprintf(why, why_cap, "%s", ok ? "ok" : w.c_str());
  return ok ? 0 : -2;
}

// Honest BLAKE3 chain of `steps` compressions (flock_chain CLI generator);
// cv0 = NULL starts from the BLAKE3 IV.
void oracle_chain_inputs(size_t steps, uint64_t seed, const uint32_t* cv0, Compression* out) {
  auto v = chain_inputs(steps, seed, cv0);
  memcpy(out, v.data(), v.size() * sizeof(Compression));
}

// Chain proof of 2^n_blocks_log compressions (ChainProofBundleLigerito bytes).
// Returns 0, -5 when cap is too small (len receives the needed size), -3 when
// the steps do not fill 2^n_blocks_log.
int oracle_prove_chain(const Compression* blocks, size_t n, int n_blocks_log, const char* domain, uint8_t* out,
                       size_t cap, size_t* len) {
  if (n != ((size_t)1 << n_blocks_log)) return -3;
  std::vector<Compression> v(blocks, blocks + n);
  uint8_t dg[32];
  digest_for(K_LOG + n_blocks_log, dg);
  ChainBundle cb = prove_chain(v, n_blocks_log, dg, domain ? domain : "flock_chain-cli");
  auto bytes = encode_chain_bundle(cb);
  *len = bytes.size();
  if (bytes.size() > cap) return -5;
  memcpy(out, bytes.data(), bytes.size());
  return 0;
}

// 0 = accepted; -1 = malformed; -2 = rejected (why gets a short reason).
int oracle_verify_chain(const uint8_t* bytes, size_t len, const char* domain, char* why, size_t why_cap) {
  ChainBundle cb;
  if (!decode_chain_bundle(bytes, len, cb)) {
    if (why && why_cap) snprintf(why, why_cap, "malformed");
    return -1;
  }
  uint8_t dg[32];
  digest_for(cb.b.params.m, dg);
  std::string w;
  bool ok = cb.b.params.m > K_LOG + 7 &&
            verify_chain(cb, cb.b.params.m, dg, mats().A, mats().B, domain ? domain : "flock_chain-cli", &w);
  if (why && why_cap) snprintf(why, why_cap, "%s", ok ? "ok" : (w.empty() ? "params" : w.c_str()));
  return ok ? 0 : -2;
}

// shift(a, b) of chain.rs:78-100 for n-coordinate points (2 u64 per element).
void oracle_shift_mle(const uint64_t* a, const uint64_t* b, int n, uint64_t* out) {
  std::vector<F128> x(n), y(n);
  for (int i = 0; i < n; i++) {
    x[i] = f128(a[2 * i], a[2 * i + 1]);
    y[i] = f128(b[2 * i], b[2 * i + 1]);
  }
  F128 r = shift_mle(x, y);
  out[0] = r.lo;
  out[1] = r.hi;
}

// F8 NTT extension S -> Lambda of one 64-bit row through the reference's
// recursive additive NTT (inverse on S = {0..63}, forward on 64 + span).
void oracle_f8_extend_ntt(uint64_t row, uint8_t* out64) {
  uint8_t v[64];
  for (int s = 0; s < 64; s++) v[s] = (uint8_t)((row >> s) & 1);
  f8_ntt_inverse(v, 6, 0);
  f8_ntt_forward(v, 6, 64);
  memcpy(out64, v, 64);
}

// Direct Lagrange extension used by the oracle's round-1 message.
void oracle_f8_extend_lagrange(uint64_t row, uint8_t* out64) {
  for (int i = 0; i < 64; i++) {
    uint8_t lam = (uint8_t)(64 + i), acc = 0;
    for (int s = 0; s < 64; s++) {
      if (!((row >> s) & 1)) continue;
      uint8_t num = 1, den = 1;
      for (int t = 0; t < 64; t++) {
        if (t == s) continue;
        num = gf8_mul(num, lam ^ (uint8_t)t);
        den = gf8_mul(den, (uint8_t)(s ^ t));
      }
      acc ^= gf8_mul(num, gf8_inv(den));
    }
    out64[i] = acc;
  }
}

}  // extern "C"

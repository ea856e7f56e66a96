// Oracle prover/verifier protocol layer (test infrastructure only).
#pragma once
#include "oracle.h"

namespace oracle {

// ---------------------------------------------------------------------------
// Fiat-Shamir transcript over BLAKE3, crates/flock-core/src/challenger.rs:183-438.
// ---------------------------------------------------------------------------
struct Transcript {
  Blake3 h;
  explicit Transcript(const std::string& domain);
  void absorb(const void* p, size_t n) { h.update(p, n); }
  void label(const std::string& s);
  void observe_f128(F128 v);
  void observe_slice(const F128* v, size_t n);
  void observe_bytes(const uint8_t* p, size_t n);
  F128 sample();
  std::vector<F128> sample_vec(size_t n);
  void state_digest(uint8_t out[32]) const;
  // challenger.rs:440-704: smallest nonce, then observe_bytes(nonce_le).
  uint64_t grind(uint32_t bits);
  bool verify_pow(uint64_t nonce, uint32_t bits);
};
bool pow_ok(const uint8_t digest[32], uint64_t nonce, uint32_t bits);

// ---------------------------------------------------------------------------
// Shared helpers.
// ---------------------------------------------------------------------------
std::vector<F128> eq_table(const std::vector<F128>& r);  // LSB-first
std::vector<F128> lagrange_s(F128 z);                    // nodes phi8(0..63)
std::vector<F128> lagrange_lambda(F128 z);               // nodes phi8(64..127)
F128 interpolate_combined(const std::vector<F128>& on_lambda, F128 z);  // zero on S
// F8 additive NTT restated from crates/flock-core/src/ntt.rs:25-170 (for tests).
void f8_ntt_forward(uint8_t* v, int k, uint8_t beta);
void f8_ntt_inverse(uint8_t* v, int k, uint8_t beta);

// ---------------------------------------------------------------------------
// Proof objects (field order = wire order, crates/flock-prover/src/proof_io.rs).
// ---------------------------------------------------------------------------
struct ZerocheckProof {
  std::vector<F128> round1_ab, round1_c;
  std::vector<std::pair<F128, F128>> rounds;
  F128 final_a, final_b, final_c;
};
struct LincheckProof {
  std::vector<std::pair<F128, F128>> rounds;
  std::vector<F128> z_partial;
};
struct LevelOpen {
  std::vector<std::vector<F128>> rows;
  std::vector<Hash32> proof;
};
struct LigeritoProof {
  Hash32 initial_root;
  LevelOpen initial;
  std::vector<Hash32> recursive_roots;
  std::vector<LevelOpen> recursive;
  std::vector<F128> yr;
  LevelOpen final_open;
  std::vector<std::pair<F128, F128>> sumcheck;  // (u_0, u_2)
  std::vector<uint64_t> grinding_nonces;
  std::vector<F128> ood_values;
  std::vector<uint64_t> fold_nonces;
};
struct Bundle {
  Hash32 root;
  PcsParams params;
  ZerocheckProof zc;
  LincheckProof lc;
  std::vector<std::vector<F128>> s_hat_v;  // ring switches
  LigeritoProof lig;
};

// Ligerito configuration for (m, profile), crates/flock-core/src/pcs/ligerito.rs:107-170, :1436-1486.
struct LigConfig {
  int initial_k = 0, yr_log_n = 0, steps = 0;
  std::vector<int> log_inv_rates, ks, queries, grinding_bits, fold_bits, ood;
};
bool ligerito_config(int m, int profile, LigConfig& out);

std::vector<uint8_t> encode_bundle(const Bundle& b);
bool decode_bundle(const uint8_t* p, size_t n, Bundle& out);

// Full prove / verify (crates/flock-prover/src/prover.rs:194-289, crates/flock-core/src/verifier.rs:53-233).
Bundle prove(const std::vector<Compression>& blocks, int n_blocks_log, const uint8_t digest[32],
             const std::string& domain = "flock-bench-v0");
bool verify(const Bundle& b, int m, const uint8_t digest[32], const SparseRows& A, const SparseRows& B,
            const std::string& domain = "flock-bench-v0", std::string* why = nullptr);

// The same with the caller's transcript (Blake3Setup::prove_fast takes
// `&mut impl Challenger`, crates/flock-prover/src/r1cs_hashes/blake3.rs:3405-3409):
// the proof continues from its state and leaves it advanced. `claim` receives
// R1csClaim { ab, c } (crates/flock-core/src/proof.rs:26-45), points in the
// RowMajor layout (crates/flock-core/src/r1cs.rs:289-334).
struct R1csClaimOut {
  F128 ab_skip, ab_value, c_skip, c_value;
  std::vector<F128> ab_inner, ab_outer, c_inner, c_outer;
};
Bundle prove_with(const std::vector<Compression>& blocks, int n_blocks_log, const uint8_t digest[32], Transcript& tr,
                  R1csClaimOut* claim);
bool verify_with(const Bundle& b, int m, const uint8_t digest[32], const SparseRows& A, const SparseRows& B,
                 Transcript& tr, std::string* why = nullptr);

// ---------------------------------------------------------------------------
// Hash-chain relation (chain.cpp; crates/flock-prover/src/chain.rs,
// r1cs_hashes/chain_common.rs, r1cs_hashes/blake3.rs:3750-3830).
// ---------------------------------------------------------------------------
struct ChainShiftProof {
  std::vector<std::pair<F128, F128>> rounds;  // (q(1), q(inf)) per round
  F128 g_at_point;
};
struct ChainClaims {
  std::vector<F128> instance_point;
  F128 sel0, value;
};
// Wire order of ChainProofBundleLigerito (proof_io.rs:152-158): hash kind,
// commitment, { zerocheck, lincheck, shift, pcs_open }, cv_0 and cv_last bits.
struct ChainBundle {
  Bundle b;
  ChainShiftProof shift;
  std::vector<uint8_t> cv0_phys, cvlast_phys;  // 256 entries, 0 or 1
};
F128 shift_mle(const std::vector<F128>& a, const std::vector<F128>& b);
ChainShiftProof prove_chain_shift(const std::vector<F128>& in_vals, const std::vector<F128>& out_vals, Transcript& tr,
                                  ChainClaims& cl);
bool verify_chain_shift(const ChainShiftProof& pf, F128 x0, F128 xlast, int n, Transcript& tr, ChainClaims& cl);
void chain_fold_io(const std::vector<F128>& z, size_t n_inst, F128 tau, std::vector<F128>& in_vals,
                   std::vector<F128>& out_vals);
std::vector<F128> chain_claim_point(F128 tau, const ChainClaims& cl);
F128 fold_public_phys(const std::vector<uint8_t>& phys, F128 tau);
std::vector<uint8_t> cv_to_phys(const uint32_t cv[8]);
std::vector<Compression> chain_inputs(size_t steps, uint64_t seed, const uint32_t cv0[8]);

// Blake3Setup::prove_chain / verify_chain (blake3.rs:3785-3830) through the
// generic chain prover (chain_common.rs:290-346, verifier :351-405).
ChainBundle prove_chain(const std::vector<Compression>& blocks, int n_blocks_log, const uint8_t digest[32],
                        const std::string& domain = "flock_chain-cli");
bool verify_chain(const ChainBundle& cb, int m, const uint8_t digest[32], const SparseRows& A, const SparseRows& B,
                  const std::string& domain = "flock_chain-cli", std::string* why = nullptr);
std::vector<uint8_t> encode_chain_bundle(const ChainBundle& cb);
bool decode_chain_bundle(const uint8_t* p, size_t n, ChainBundle& out);

}  // namespace oracle

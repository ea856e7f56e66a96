// CPU oracle for the flock BLAKE3-compression prover hot path.
//
// TEST INFRASTRUCTURE ONLY. This is a plain C++ restatement of the reference
// Rust prover (Layr-Labs/flock-challenge) used to check the CUDA product path
// bit for bit. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg may load it; the product library never links or calls it.
//
// Each routine cites the reference file:line it restates. Paths are relative to
// the reference project root.
#pragma once
#include <cstddef>
#include <cstdint>
#include <array>
#include <string>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------------------
// GF(2^128), polynomial basis, modulus x^128 + x^7 + x^2 + x + 1.
// crates/flock-core/src/field/gf2_128.rs:22-135, :192-216; portable.rs:4-38
// ---------------------------------------------------------------------------
struct F128 {
  uint64_t lo = 0, hi = 0;
  bool operator==(const F128& o) const { return lo == o.lo && hi == o.hi; }
  bool operator!=(const F128& o) const { return !(*this == o); }
  F128 operator+(const F128& o) const { return {lo ^ o.lo, hi ^ o.hi}; }
  F128& operator+=(const F128& o) { lo ^= o.lo; hi ^= o.hi; return *this; }
  bool is_zero() const { return (lo | hi) == 0; }
};
inline F128 f128(uint64_t lo, uint64_t hi = 0) { F128 r; r.lo = lo; r.hi = hi; return r; }
F128 gf_mul(F128 a, F128 b);
F128 gf_mul_portable(F128 a, F128 b);  // same value, portable integer code on every host
int gf_mul_uses_pmull();               // 1 when gf_mul runs on the Arm PMULL instruction
F128 gf_inv(F128 a);
F128 gf_mul_x(F128 a);
inline F128 operator*(F128 a, F128 b) { return gf_mul(a, b); }

// GF(2^8), AES modulus 0x11B, and the field embedding phi8: GF(2^8) -> GF(2^128)
// (crates/flock-core/src/field/gf2_8.rs:1-60, field/phi8.rs:1-30).
uint8_t gf8_mul(uint8_t a, uint8_t b);
uint8_t gf8_inv(uint8_t a);
F128 phi8(uint8_t v);

// ---------------------------------------------------------------------------
// BLAKE3 (public specification; the reference calls the un-vendored `blake3`
// 1.8.5 crate) plus the reference's own compression restatement at
// crates/flock-prover/src/r1cs_hashes/blake3.rs:271-310.
// ---------------------------------------------------------------------------
extern const uint32_t B3_IV[8];
enum : uint32_t { B3_CHUNK_START = 1, B3_CHUNK_END = 2, B3_PARENT = 4, B3_ROOT = 8 };
void b3_compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                 uint32_t block_len, uint32_t flags, uint32_t out[16]);

struct Blake3 {
  // Incremental hasher with a chaining-value stack (spec section 5.1.2).
  uint32_t cv[8];
  uint8_t buf[64];
  size_t buf_len = 0;
  size_t blocks_in_chunk = 0;  // compressed blocks in the current chunk
  uint64_t chunk_counter = 0;
  std::vector<std::array<uint32_t, 8>> stack;
  Blake3();
  void update(const void* data, size_t len);
  // 32-byte root hash.
  void finalize(uint8_t out[32]) const;
  // Root output bytes of arbitrary length (XOF).
  void finalize_xof(uint8_t* out, size_t len) const;
  // Chaining value of the root node without the ROOT flag.
  void finalize_non_root(uint8_t out[32]) const;

 private:
  struct Output { uint32_t cv[8]; uint32_t block[16]; uint64_t counter; uint32_t len; uint32_t flags; };
  Output final_output() const;
};
void b3_hash(const void* data, size_t len, uint8_t out[32]);
void b3_parent_cv(const uint8_t left[32], const uint8_t right[32], uint8_t out[32]);

// ---------------------------------------------------------------------------
// Inputs and witness.
// ---------------------------------------------------------------------------
struct Compression {
  uint32_t cv[8];
  uint32_t m[16];
  uint64_t counter;
  uint32_t block_len;
  uint32_t flags;
};
// benchmark-tools/common/src/lib.rs:20-33
std::vector<Compression> generate_compressions(uint32_t log2_size, uint64_t seed);
// crates/flock-prover/src/r1cs_hashes/blake3.rs:4910-4930 (canary / benches input)
std::vector<Compression> canary_compressions(uint32_t log2_size);

constexpr int K_LOG = 14;
constexpr int K = 1 << K_LOG;
constexpr int K_SKIP = 6;
constexpr int USEFUL_BITS = 15409;
constexpr int Z_CONST_POS = 512;

// n_blocks_log for n compressions (blake3.rs:1080-1084).
int min_n_blocks_log(size_t n);

// Packed (z, a, b) witness, 2^(m-7) F128 each, plus the lincheck byte stripe
// (2^m / 8 bytes). Padding slots hold the compression of the all-zero input.
// blake3.rs:965-1076, :1124-1290, :2928-3180; r1cs_hashes/common.rs:85-101.
struct Witness {
  int m = 0;
  std::vector<F128> z, a, b;
  std::vector<uint8_t> stripe;
};
Witness build_witness(const std::vector<Compression>& blocks, int n_blocks_log, bool with_stripe = true);

// Sparse base matrices (blake3.rs:485-631) and the statement digest
// (crates/flock-core/src/r1cs.rs:343-365, :431-460).
struct SparseRows {
  std::vector<std::vector<uint32_t>> rows;
};
void build_matrices(SparseRows& a0, SparseRows& b0);
void statement_digest(int m, const SparseRows& a0, const SparseRows& b0, uint8_t out[32]);

// ---------------------------------------------------------------------------
// Additive NTT over GF(2^128), standard basis {1, x, x^2, ...}.
// crates/flock-core/src/ntt/additive_ntt_f128.rs:57-129, :514-552, :1281-1312
// ---------------------------------------------------------------------------
struct NttF128 {
  int log_d = 0;
  std::vector<F128> twiddles;  // breadth-first, layer l at offset 2^l - 1
  explicit NttF128(int dim);
  F128 twiddle(int layer, size_t block) const { return twiddles[((size_t)1 << layer) - 1 + block]; }
  // Interleaved SoA forward transform data[pos*num_ntts + lane] from start_layer.
  void forward_interleaved(F128* data, size_t n_total, size_t num_ntts, int start_layer) const;
};

// ---------------------------------------------------------------------------
// Merkle (BLAKE3 tree semantics), crates/flock-core/src/merkle.rs:200-235, :706-1004
// ---------------------------------------------------------------------------
struct Hash32 {
  uint8_t b[32];
  bool operator==(const Hash32& o) const;
};
Hash32 leaf_cv(const uint8_t* data, size_t len);
Hash32 parent_cv(const Hash32& l, const Hash32& r);
// Flat tree: leaves first, each level appended, root last (2*n_leaves-1 nodes).
std::vector<Hash32> merkle_tree(const uint8_t* data, size_t len, size_t n_leaves);
std::vector<Hash32> merkle_multi_proof(const std::vector<Hash32>& tree, size_t n_leaves,
                                       std::vector<size_t> positions);
bool verify_merkle_multi_proof(const Hash32& root, size_t n_leaves, const std::vector<size_t>& pos,
                               const std::vector<Hash32>& leaf_hashes, const std::vector<Hash32>& proof);

// ---------------------------------------------------------------------------
// PCS commit, crates/flock-core/src/pcs/commit.rs:32-92, :250-473, :691-818
// ---------------------------------------------------------------------------
struct PcsParams {
  int m = 0;
  int log_inv_rate = 1;
  int log_batch_size = 6;
  int profile = 0;      // LigeritoProfile::Fast
  int merkle_hash = 1;  // HashKind::Blake3
  int log_msg_len() const { return m - 7; }
  int log_dim() const { return log_msg_len() - log_batch_size; }
  int k_code() const { return log_dim() + log_inv_rate; }
  size_t n_positions() const { return (size_t)1 << k_code(); }
  size_t num_ntts() const { return (size_t)1 << log_batch_size; }
};
struct CommitData {
  std::vector<F128> codeword;
  std::vector<Hash32> tree;
  Hash32 root() const { return tree.back(); }
};
CommitData commit(const std::vector<F128>& z, const PcsParams& p);

}  // namespace oracle

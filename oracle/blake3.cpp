// BLAKE3 for the oracle (test infrastructure only).
//
// The compression function follows the reference's own restatement at
// crates/flock-prover/src/r1cs_hashes/blake3.rs:271-310 (IV, message
// permutation, G schedule, finalization XORs). The chunk/tree modes follow the
// public BLAKE3 specification (the reference reaches them through the
// un-vendored `blake3` 1.8.5 crate at crates/flock-core/src/merkle.rs:200-210
// and challenger.rs:240-360).
#include <cstring>

#include "oracle.h"

namespace oracle {

const uint32_t B3_IV[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                           0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
static const int B3_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

static inline void g(uint32_t* s, int a, int b, int c, int d, uint32_t mx, uint32_t my) {
  s[a] = s[a] + s[b] + mx;
  s[d] = rotr(s[d] ^ s[a], 16);
  s[c] = s[c] + s[d];
  s[b] = rotr(s[b] ^ s[c], 12);
  s[a] = s[a] + s[b] + my;
  s[d] = rotr(s[d] ^ s[a], 8);
  s[c] = s[c] + s[d];
  s[b] = rotr(s[b] ^ s[c], 7);
}

void b3_compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                 uint32_t block_len, uint32_t flags, uint32_t out[16]) {
  uint32_t s[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    B3_IV[0], B3_IV[1], B3_IV[2], B3_IV[3],
                    (uint32_t)counter, (uint32_t)(counter >> 32), block_len, flags};
  uint32_t m[16];
  memcpy(m, block, 64);
  for (int r = 0; r < 7; r++) {
    g(s, 0, 4, 8, 12, m[0], m[1]);
    g(s, 1, 5, 9, 13, m[2], m[3]);
    g(s, 2, 6, 10, 14, m[4], m[5]);
    g(s, 3, 7, 11, 15, m[6], m[7]);
    g(s, 0, 5, 10, 15, m[8], m[9]);
    g(s, 1, 6, 11, 12, m[10], m[11]);
    g(s, 2, 7, 8, 13, m[12], m[13]);
    g(s, 3, 4, 9, 14, m[14], m[15]);
    if (r < 6) {
      uint32_t t[16];
      for (int i = 0; i < 16; i++) t[i] = m[B3_PERM[i]];
      memcpy(m, t, 64);
    }
  }
  for (int i = 0; i < 8; i++) {
    out[i] = s[i] ^ s[i + 8];
    out[i + 8] = s[i + 8] ^ cv[i];
  }
}

static void words_from_bytes(const uint8_t* b, size_t len, uint32_t w[16]) {
  uint8_t tmp[64] = {0};
  memcpy(tmp, b, len);
  for (int i = 0; i < 16; i++)
    w[i] = (uint32_t)tmp[4 * i] | ((uint32_t)tmp[4 * i + 1] << 8) | ((uint32_t)tmp[4 * i + 2] << 16) |
           ((uint32_t)tmp[4 * i + 3] << 24);
}
static void bytes_from_words(const uint32_t* w, int n, uint8_t* out) {
  for (int i = 0; i < n; i++) {
    out[4 * i] = (uint8_t)w[i];
    out[4 * i + 1] = (uint8_t)(w[i] >> 8);
    out[4 * i + 2] = (uint8_t)(w[i] >> 16);
    out[4 * i + 3] = (uint8_t)(w[i] >> 24);
  }
}

Blake3::Blake3() { memcpy(cv, B3_IV, 32); }

void Blake3::update(const void* data, size_t len) {
  const uint8_t* p = (const uint8_t*)data;
  while (len > 0) {
    // A completed chunk (16 blocks, the last still buffered) is closed only
    // once more input arrives, so the final chunk can take the ROOT flag.
    if (blocks_in_chunk == 15 && buf_len == 64) {
      uint32_t w[16], out[16];
      words_from_bytes(buf, 64, w);
      b3_compress(cv, w, chunk_counter, 64, B3_CHUNK_END, out);
      std::array<uint32_t, 8> ncv;
      memcpy(ncv.data(), out, 32);
      uint64_t total = chunk_counter + 1;
      while ((total & 1) == 0) {
        uint32_t blk[16];
        memcpy(blk, stack.back().data(), 32);
        memcpy(blk + 8, ncv.data(), 32);
        stack.pop_back();
        b3_compress(B3_IV, blk, 0, 64, B3_PARENT, out);
        memcpy(ncv.data(), out, 32);
        total >>= 1;
      }
      stack.push_back(ncv);
      chunk_counter++;
      memcpy(cv, B3_IV, 32);
      blocks_in_chunk = 0;
      buf_len = 0;
    }
    if (buf_len == 64) {
      uint32_t w[16], out[16];
      words_from_bytes(buf, 64, w);
      b3_compress(cv, w, chunk_counter, 64, blocks_in_chunk == 0 ? B3_CHUNK_START : 0, out);
      memcpy(cv, out, 32);
      blocks_in_chunk++;
      buf_len = 0;
    }
    size_t take = 64 - buf_len;
    if (take > len) take = len;
    memcpy(buf + buf_len, p, take);
    buf_len += take;
    p += take;
    len -= take;
  }
}

Blake3::Output Blake3::final_output() const {
  Output o;
  memcpy(o.cv, cv, 32);
  words_from_bytes(buf, buf_len, o.block);
  o.counter = chunk_counter;
  o.len = (uint32_t)buf_len;
  o.flags = B3_CHUNK_END | (blocks_in_chunk == 0 ? B3_CHUNK_START : 0);
  for (size_t i = stack.size(); i-- > 0;) {
    uint32_t out[16];
    b3_compress(o.cv, o.block, o.counter, o.len, o.flags, out);
    Output p;
    memcpy(p.cv, B3_IV, 32);
    memcpy(p.block, stack[i].data(), 32);
    memcpy(p.block + 8, out, 32);
    p.counter = 0;
    p.len = 64;
    p.flags = B3_PARENT;
    o = p;
  }
  return o;
}

void Blake3::finalize(uint8_t out[32]) const { finalize_xof(out, 32); }

void Blake3::finalize_xof(uint8_t* out, size_t len) const {
  Output o = final_output();
  uint64_t ctr = 0;
  while (len > 0) {
    uint32_t w[16];
    uint8_t blk[64];
    b3_compress(o.cv, o.block, ctr, o.len, o.flags | B3_ROOT, w);
    bytes_from_words(w, 16, blk);
    size_t take = len < 64 ? len : 64;
    memcpy(out, blk, take);
    out += take;
    len -= take;
    ctr++;
  }
}

void Blake3::finalize_non_root(uint8_t out[32]) const {
  Output o = final_output();
  uint32_t w[16];
  b3_compress(o.cv, o.block, o.counter, o.len, o.flags, w);
  bytes_from_words(w, 8, out);
}

void b3_hash(const void* data, size_t len, uint8_t out[32]) {
  Blake3 h;
  h.update(data, len);
  h.finalize(out);
}

void b3_parent_cv(const uint8_t left[32], const uint8_t right[32], uint8_t out[32]) {
  uint8_t blk[64];
  memcpy(blk, left, 32);
  memcpy(blk + 32, right, 32);
  uint32_t w[16], o[16];
  words_from_bytes(blk, 64, w);
  b3_compress(B3_IV, w, 0, 64, B3_PARENT, o);
  bytes_from_words(o, 8, out);
}

}  // namespace oracle

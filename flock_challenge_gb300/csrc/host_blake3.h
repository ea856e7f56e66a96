// Host BLAKE3 (public specification) for the Fiat-Shamir transcript and the
// statement digest. Incremental chunk state plus chaining-value stack; the
// root output is extendable (XOF). Matches the device compression in
// blake3.cuh word for word.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

namespace hb3 {

static constexpr uint32_t IV[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                   0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
enum : uint32_t { CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8 };

inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

inline void compress(const uint32_t cv[8], const uint32_t m_in[16], uint64_t ctr, uint32_t len, uint32_t flags,
                     uint32_t out[16]) {
  static const int P[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
  uint32_t v[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    IV[0], IV[1], IV[2], IV[3], (uint32_t)ctr, (uint32_t)(ctr >> 32), len, flags};
  uint32_t m[16];
  memcpy(m, m_in, 64);
  auto g = [&](int a, int b, int c, int d, uint32_t x, uint32_t y) {
    v[a] += v[b] + x; v[d] = rotr(v[d] ^ v[a], 16);
    v[c] += v[d];     v[b] = rotr(v[b] ^ v[c], 12);
    v[a] += v[b] + y; v[d] = rotr(v[d] ^ v[a], 8);
    v[c] += v[d];     v[b] = rotr(v[b] ^ v[c], 7);
  };
  for (int r = 0; r < 7; r++) {
    g(0, 4, 8, 12, m[0], m[1]); g(1, 5, 9, 13, m[2], m[3]);
    g(2, 6, 10, 14, m[4], m[5]); g(3, 7, 11, 15, m[6], m[7]);
    g(0, 5, 10, 15, m[8], m[9]); g(1, 6, 11, 12, m[10], m[11]);
    g(2, 7, 8, 13, m[12], m[13]); g(3, 4, 9, 14, m[14], m[15]);
    uint32_t t[16];
    for (int i = 0; i < 16; i++) t[i] = m[P[i]];
    memcpy(m, t, 64);
  }
  for (int i = 0; i < 8; i++) {
    out[i] = v[i] ^ v[i + 8];
    out[i + 8] = v[i + 8] ^ cv[i];
  }
}

inline void load_words(const uint8_t* b, size_t n, uint32_t w[16]) {
  uint8_t t[64] = {0};
  memcpy(t, b, n);
  for (int i = 0; i < 16; i++) w[i] = t[4 * i] | (t[4 * i + 1] << 8) | (t[4 * i + 2] << 16) | ((uint32_t)t[4 * i + 3] << 24);
}

class Hasher {
 public:
  Hasher() { memcpy(cv_, IV, 32); }

  void update(const void* data, size_t n) {
    const uint8_t* p = (const uint8_t*)data;
    while (n) {
      if (buf_len_ == 64 && blocks_ == 15) close_chunk();
      if (buf_len_ == 64) {
        uint32_t w[16], o[16];
        load_words(buf_, 64, w);
        compress(cv_, w, chunk_, 64, blocks_ == 0 ? CHUNK_START : 0, o);
        memcpy(cv_, o, 32);
        blocks_++;
        buf_len_ = 0;
      }
      size_t take = 64 - buf_len_;
      if (take > n) take = n;
      memcpy(buf_ + buf_len_, p, take);
      buf_len_ += take;
      p += take;
      n -= take;
    }
  }

  // Root output bytes (XOF) of the current state; the state is unchanged.
  void xof(uint8_t* out, size_t n) const {
    Node o = root_node();
    for (uint64_t ctr = 0; n; ctr++) {
      uint32_t w[16];
      compress(o.cv, o.block, ctr, o.len, o.flags | ROOT, w);
      size_t take = n < 64 ? n : 64;
      memcpy(out, w, take);  // little-endian host
      out += take;
      n -= take;
    }
  }
  void finalize(uint8_t out[32]) const { xof(out, 32); }

 private:
  struct Node {
    uint32_t cv[8], block[16];
    uint64_t ctr;
    uint32_t len, flags;
  };
  void close_chunk() {
    uint32_t w[16], o[16];
    load_words(buf_, 64, w);
    compress(cv_, w, chunk_, 64, CHUNK_END, o);
    std::vector<uint32_t> ncv(o, o + 8);
    for (uint64_t total = chunk_ + 1; (total & 1) == 0; total >>= 1) {
      uint32_t blk[16];
      memcpy(blk, stack_.back().data(), 32);
      memcpy(blk + 8, ncv.data(), 32);
      stack_.pop_back();
      compress(IV, blk, 0, 64, PARENT, o);
      ncv.assign(o, o + 8);
    }
    stack_.push_back(ncv);
    chunk_++;
    memcpy(cv_, IV, 32);
    blocks_ = 0;
    buf_len_ = 0;
  }
  Node root_node() const {
    Node o;
    memcpy(o.cv, cv_, 32);
    load_words(buf_, buf_len_, o.block);
    o.ctr = chunk_;
    o.len = (uint32_t)buf_len_;
    o.flags = CHUNK_END | (blocks_ == 0 ? CHUNK_START : 0);
    for (size_t i = stack_.size(); i-- > 0;) {
      uint32_t w[16];
      compress(o.cv, o.block, o.ctr, o.len, o.flags, w);
      Node p;
      memcpy(p.cv, IV, 32);
      memcpy(p.block, stack_[i].data(), 32);
      memcpy(p.block + 8, w, 32);
      p.ctr = 0;
      p.len = 64;
      p.flags = PARENT;
      o = p;
    }
    return o;
  }

  uint32_t cv_[8];
  uint8_t buf_[64];
  size_t buf_len_ = 0, blocks_ = 0;
  uint64_t chunk_ = 0;
  std::vector<std::vector<uint32_t>> stack_;
};

}  // namespace hb3

// Fiat-Shamir transcript of the prover, kept on the host.
//
// Byte format of crates/flock-core/src/challenger.rs:183-438 (FsChallenger
// over BLAKE3): every operation appends to one running BLAKE3 input stream
//   domain  0x01 || len_le64 || bytes      label 0x02 || len_le64 || bytes
//   f128    0x03 0x01 || lo_le || hi_le     slice 0x03 0x02 || n_le64 || elems
//   bytes   0x05 || len_le64 || bytes
//   sample  0x04 0x01, then 16 XOF bytes of the current state, re-absorbed
//   vector  0x04 0x02 || n_le64, then 16n XOF bytes, re-absorbed
// The PoW pre-image is state_digest || nonce_le || 0^24 (challenger.rs:1246-1296).
#pragma once
#include <string>
#include <vector>

#include "host_blake3.h"
#include "host_field.h"

namespace fs {

class Transcript {
 public:
  explicit Transcript(const std::string& domain) {
    uint8_t op = 0x01;
    h_.update(&op, 1);
    put_len(domain.size());
    h_.update(domain.data(), domain.size());
  }
  void label(const char* s) { label(s, strlen(s)); }
  void label(const void* s, size_t n) {
    uint8_t op = 0x02;
    h_.update(&op, 1);
    put_len(n);
    h_.update(s, n);
  }
  void observe(hf::F v) {
    uint8_t b[18] = {0x03, 0x01};
    memcpy(b + 2, &v.lo, 8);
    memcpy(b + 10, &v.hi, 8);
    h_.update(b, 18);
  }
  void observe_slice(const hf::F* v, size_t n) {
    uint8_t b[2] = {0x03, 0x02};
    h_.update(b, 2);
    put_len(n);
    h_.update(v, 16 * n);
  }
  void observe_bytes(const void* p, size_t n) {
    uint8_t op = 0x05;
    h_.update(&op, 1);
    put_len(n);
    h_.update(p, n);
  }
  hf::F sample() {
    uint8_t b[2] = {0x04, 0x01};
    h_.update(b, 2);
    hf::F r;
    h_.xof(reinterpret_cast<uint8_t*>(&r), 16);
    h_.update(&r, 16);
    return r;
  }
  std::vector<hf::F> sample_vec(size_t n) {
    uint8_t b[2] = {0x04, 0x02};
    h_.update(b, 2);
    put_len(n);
    std::vector<hf::F> v(n);
    if (n) {
      h_.xof(reinterpret_cast<uint8_t*>(v.data()), 16 * n);
      h_.update(v.data(), 16 * n);
    }
    return v;
  }
  void digest(uint8_t out[32]) const { h_.finalize(out); }
  void absorb_nonce(uint64_t nonce) { observe_bytes(&nonce, 8); }

 private:
  void put_len(uint64_t n) { h_.update(&n, 8); }
  hb3::Hasher h_;
};

}  // namespace fs

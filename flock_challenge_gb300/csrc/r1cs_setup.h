// Setup-time R1CS data (see r1cs_setup.cpp).
#pragma once
#include <cstdint>
#include <vector>

struct HostCsc {
  std::vector<uint32_t> a_ptr, a_idx, b_ptr, b_idx;  // column pointers / row indices
};

// BLAKE3 statement digest of the BLAKE3 R1CS instance with 2^(m-14) blocks; cached per m.
void flock_statement_digest(int m, uint8_t out[32]);
// Column-major copies of A_0 and B_0 (built once).
const HostCsc& flock_host_csc();

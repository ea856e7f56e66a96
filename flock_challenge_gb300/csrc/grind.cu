// Proof-of-work grind (crates/flock-core/src/challenger.rs:440-704, :1246-1310).
//
// The nonce is the smallest n >= 0 whose BLAKE3 hash of the 64-byte pre-image
// digest || n_le64 || 0^24 (one block, CHUNK_START | CHUNK_END | ROOT) has at
// least `bits` leading zero bits, read MSB-first from byte 0. Each thread
// tests one nonce of a window and lowers a device minimum with atomicMin; the
// host scans windows in increasing order and stops at the first window with a
// hit, so the result is the global minimum. Grinds of a few bits (about 2^bits
// hashes) are cheaper on the host than a launch and a wait: they test the
// nonces in increasing order there.
#include <cstring>

#include "blake3.cuh"
#include "flock_internal.h"
#include "host_blake3.h"

namespace {

__device__ __forceinline__ bool leading_zeros_ok(const uint32_t h[8], uint32_t bits) {
  // byte k of the hash is byte (k & 3) of word k >> 2 (little-endian words)
  for (uint32_t k = 0; k < 32 && bits > 0; k++) {
    uint32_t byte = (h[k >> 2] >> (8 * (k & 3))) & 255;
    if (bits >= 8) {
      if (byte) return false;
      bits -= 8;
    } else {
      return (byte >> (8 - bits)) == 0;
    }
  }
  return true;
}

struct Digest {
  uint32_t w[8];
};

// `other` (may be null): the other result slot, reset here for the next grind
// (which runs after this launch in stream order), so no grind needs a memset.
__global__ void grind_kernel(const __grid_constant__ Digest digest, uint64_t start, uint64_t count, uint32_t bits,
                             unsigned long long* __restrict__ best, unsigned long long* __restrict__ other) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  if (other && i == 0) *other = ~0ull;
  uint64_t nonce = start + i;
  uint32_t m[16];
#pragma unroll
  for (int k = 0; k < 8; k++) m[k] = digest.w[k];
  m[8] = (uint32_t)nonce;
  m[9] = (uint32_t)(nonce >> 32);
#pragma unroll
  for (int k = 10; k < 16; k++) m[k] = 0;
  uint32_t cv[8];
#pragma unroll
  for (int k = 0; k < 8; k++) cv[k] = b3::IV(k);
  b3::compress_cv(cv, m, 64, b3::CHUNK_START | b3::CHUNK_END | b3::ROOT);
  if (leading_zeros_ok(cv, bits)) atomicMin(best, (unsigned long long)nonce);
}

// Grinds of at most this many bits run on the host: about 2^bits hashes of
// ~0.1 us each against a kernel launch and a wait for its result (~13 us of
// idle device per grind).
constexpr uint32_t kHostGrindBits = 6;

bool host_pow(const uint32_t dg[8], uint64_t nonce, uint32_t bits) {
  uint32_t m[16] = {0}, o[16];
  for (int k = 0; k < 8; k++) m[k] = dg[k];
  m[8] = (uint32_t)nonce;
  m[9] = (uint32_t)(nonce >> 32);
  hb3::compress(hb3::IV, m, 0, 64, hb3::CHUNK_START | hb3::CHUNK_END | hb3::ROOT, o);
  for (uint32_t k = 0; k < 32 && bits > 0; k++) {
    const uint32_t byte = (o[k >> 2] >> (8 * (k & 3))) & 255;
    if (bits >= 8) {
      if (byte) return false;
      bits -= 8;
    } else {
      return (byte >> (8 - bits)) == 0;
    }
  }
  return true;
}

}  // namespace

// Returns the smallest satisfying nonce. d_scratch: >= 16 bytes of device
// memory, two result slots; h_best: 8 bytes of host memory the window result
// is read into (pinned memory keeps the read cheap). The digest travels as a
// kernel argument, so nothing is copied to the device. With `parity` (a
// caller's counter; the slots set to all ones before its first grind), the
// grinds alternate slots and each resets the other one for the next; without,
// the slot is cleared by a memset first.
int flock_grind(const uint8_t digest[32], uint32_t bits, void* d_scratch, int* parity, uint64_t* h_best,
                cudaStream_t st, WaitStats* waits, uint64_t* nonce) {
  if (bits == 0) {
    *nonce = 0;
    return FLOCK_OK;
  }
  if (bits > 60) return FLOCK_ERR_SHAPE;
  Digest dg;
  memcpy(dg.w, digest, 32);
  if (bits <= kHostGrindBits) {
    // in increasing order, as the windows below; the result slots are left
    // alone, so the alternation of the device grinds is unchanged
    for (uint64_t n = 0; n < ((uint64_t)1 << 20); n++)
      if (host_pow(dg.w, n, bits)) {
        *nonce = n;
        return FLOCK_OK;
      }
  }
  unsigned long long* d_best = (unsigned long long*)d_scratch;
  unsigned long long* d_other = nullptr;
  if (parity) {
    d_best += *parity & 1;
    d_other = (unsigned long long*)d_scratch + ((*parity & 1) ^ 1);
    ++*parity;
  }
  const unsigned long long none = ~0ull;
  if (!parity && cudaMemsetAsync(d_best, 0xFF, 8, st) != cudaSuccess) return FLOCK_ERR_CUDA;
  // About two expected hits per window: a miss costs one more window, an
  // oversized window wastes work on every grind (most grinds are 2..14 bits).
  int wlog = (int)bits + 1;
  if (wlog < 12) wlog = 12;
  if (wlog > 26) wlog = 26;
  uint64_t window = (uint64_t)1 << wlog;
  for (uint64_t start = 0;; start += window) {
    grind_kernel<<<(unsigned)((window + 255) / 256), 256, 0, st>>>(dg, start, window, bits, d_best, d_other);
    flock_count_launch();
    if (cudaGetLastError() != cudaSuccess) return FLOCK_ERR_CUDA;
    if (cudaMemcpyAsync(h_best, d_best, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return FLOCK_ERR_CUDA;
    const cudaError_t we = flock_stream_wait(st, waits);
    if (we != cudaSuccess) return we == cudaErrorTimeout ? FLOCK_ERR_TIMEOUT : FLOCK_ERR_CUDA;
    if (*h_best != none) {
      *nonce = *h_best;
      return FLOCK_OK;
    }
    if (start > ((uint64_t)1 << 62)) return FLOCK_ERR_TIMEOUT;
  }
}

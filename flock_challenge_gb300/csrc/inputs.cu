// Benchmark input generator on the device.
//
// benchmark-tools/common/src/lib.rs:20-33: a SplitMix64 stream seeded with
// seed ^ rotl(log2, 29); each compression takes 25 consecutive draws (8 cv
// words, 16 message words, one counter word; each draw keeps the low 32 bits),
// with block_len 64 and flags 11. SplitMix64's state after k steps is
// state0 + k * 0x9E3779B97F4A7C15, so draw k is a pure function of k and every
// thread generates its compression independently.
#include "flock_internal.h"

namespace {

__device__ __forceinline__ uint32_t splitmix_draw(uint64_t state0, uint64_t k) {
  uint64_t z = state0 + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return (uint32_t)(z ^ (z >> 31));
}

__global__ void gen_inputs_kernel(uint64_t state0, size_t n, flock_compression* __restrict__ out) {
  size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  uint64_t k = (uint64_t)j * 25;
  flock_compression c;
#pragma unroll
  for (int i = 0; i < 8; i++) c.cv[i] = splitmix_draw(state0, k + i);
#pragma unroll
  for (int i = 0; i < 16; i++) c.m[i] = splitmix_draw(state0, k + 8 + i);
  c.counter = splitmix_draw(state0, k + 24);
  c.block_len = 64;
  c.flags = 11;
  out[j] = c;
}

}  // namespace

int flock_launch_gen_inputs(uint64_t state0, size_t n, void* d_out, cudaStream_t st) {
  if (n == 0) return FLOCK_OK;
  gen_inputs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(state0, n, (flock_compression*)d_out);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

// BLAKE3 R1CS witness generation: one thread per compression.
//
// Restates the witness of crates/flock-prover/src/r1cs_hashes/blake3.rs:965-1076
// and its packed (z, a, b) writer at :1124-1290 (r1cs_hashes/common.rs:85-101):
// per compression a 2^14-bit block in the layout of blake3.rs:107-231
//   [0,256) cv | [256,512) out_lo | 512 const | [513,1025) m | t_lo | t_hi |
//   block_len | flags | 56 G-blocks x 250 bits | [15153,15409) out_hi | zeros
// For a carry-only ADD x + y with cin = (x + y) ^ x ^ y, bits 0..30 hold
// z = (x^cin)&(y^cin), a = x^cin, b = y^cin; input and lin-id words hold
// z = a = value, b = all ones; the constant bit is (1,1,1); c = z.
// It also writes the lincheck byte stripe of crates/flock-core/src/lincheck.rs:88-110:
// byte (j/8)*2^14 + i has bit (j%8) = witness bit i of compression j.
//
// Threads run the data-independent BLAKE3 schedule in lockstep, so every lane
// completes witness word w at the same instruction. Completed 64-bit words are
// staged per warp in shared memory and written out 16 words at a time as
// 128-byte runs per compression; the stripe bytes of each group of eight
// compressions are produced from the same staging by 8x8 bit transposes.
#include <cstdint>

#include "blake3.cuh"
#include "flock_internal.h"

namespace {

constexpr int STAGE_WORDS = 16;
constexpr int STAGE_STRIDE = STAGE_WORDS + 1;  // 64-bit words; avoids bank conflicts
constexpr int WARPS_PER_BLOCK = 4;
constexpr int KWORDS = 256;  // 64-bit words per compression block

struct WarpCtx {
  uint64_t* sz;  // [32][STAGE_STRIDE]
  uint64_t* sa;
  uint64_t* sb;
  uint64_t* gz;
  uint64_t* ga;
  uint64_t* gb;
  uint8_t* stripe;
  size_t warp_slot0;  // first compression slot of this warp
  int n_valid;        // valid lanes in this warp (slots < n_total)
  int lane;
};

__device__ __forceinline__ uint64_t transpose8x8(uint64_t x) {
  uint64_t t;
  t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull; x = x ^ t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull; x = x ^ t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull; x = x ^ t ^ (t << 28);
  return x;
}

// Writes the 16 staged words (global word index w0..w0+15) of all lanes.
// (Scalar arguments, so the call passes them in registers; the context
// struct itself never has to live in memory.)
__device__ __noinline__ void flush_words(uint64_t* sz, uint64_t* gz, uint64_t* ga, uint64_t* gb, uint8_t* stripe,
                                        size_t warp_slot0, int n_valid, int lane, int w0) {
  struct {
    uint64_t *sz, *sa, *sb, *gz, *ga, *gb;
    uint8_t* stripe;
    size_t warp_slot0;
    int n_valid, lane;
  } c = {sz, sz + 32 * STAGE_STRIDE, sz + 64 * STAGE_STRIDE, gz, ga, gb, stripe, warp_slot0, n_valid, lane};
  __syncwarp();
  const int half = c.lane >> 4, j = c.lane & 15;
#pragma unroll 4
  for (int i = 0; i < 16; i++) {
    int comp = 2 * i + half;
    if (comp < c.n_valid) {
      size_t g = (c.warp_slot0 + comp) * KWORDS + w0 + j;
      c.gz[g] = c.sz[comp * STAGE_STRIDE + j];
      if (c.ga) {
        c.ga[g] = c.sa[comp * STAGE_STRIDE + j];
        c.gb[g] = c.sb[comp * STAGE_STRIDE + j];
      }
    }
  }
  if (c.stripe) {
    // 4 groups of 8 compressions x 16 words; two items per lane.
#pragma unroll
    for (int k = 0; k < 2; k++) {
      int item = c.lane + 32 * k;
      int grp = item >> 4, w = item & 15;
      if (8 * grp < c.n_valid) {
        uint64_t r8[8];
#pragma unroll
        for (int r = 0; r < 8; r++) r8[r] = c.sz[(8 * grp + r) * STAGE_STRIDE + w];
        uint64_t outw[8];
#pragma unroll
        for (int p = 0; p < 8; p++) {
          uint64_t x = 0;
#pragma unroll
          for (int r = 0; r < 8; r++) x |= ((r8[r] >> (8 * p)) & 0xFFull) << (8 * r);
          outw[p] = transpose8x8(x);
        }
        size_t byte_idx = (c.warp_slot0 >> 3) + grp;
        uint4* dst = reinterpret_cast<uint4*>(c.stripe + byte_idx * (size_t)FLOCK_K + (size_t)(w0 + w) * 64);
#pragma unroll
        for (int q = 0; q < 4; q++)
          dst[q] = make_uint4((uint32_t)outw[2 * q], (uint32_t)(outw[2 * q] >> 32), (uint32_t)outw[2 * q + 1],
                              (uint32_t)(outw[2 * q + 1] >> 32));
      }
    }
  }
  __syncwarp();
}

struct Sink {
  uint64_t pz, pa, pb;
  int used;
  int word;
  __device__ __forceinline__ void emit(const WarpCtx& c, uint64_t z, uint64_t a, uint64_t b) {
    int j = word % STAGE_WORDS;
    c.sz[c.lane * STAGE_STRIDE + j] = z;
    c.sa[c.lane * STAGE_STRIDE + j] = a;
    c.sb[c.lane * STAGE_STRIDE + j] = b;
    word++;
    if (word % STAGE_WORDS == 0)
      flush_words(c.sz, c.gz, c.ga, c.gb, c.stripe, c.warp_slot0, c.n_valid, c.lane, word - STAGE_WORDS);
  }
  // Appends `width` bits (values already masked to width).
  __device__ __forceinline__ void push(const WarpCtx& c, uint32_t z, uint32_t a, uint32_t b, int width) {
    pz |= (uint64_t)z << used;
    pa |= (uint64_t)a << used;
    pb |= (uint64_t)b << used;
    if (used + width >= 64) {
      emit(c, pz, pa, pb);
      int sh = 64 - used;
      pz = sh >= 32 ? 0 : ((uint64_t)z >> sh);
      pa = sh >= 32 ? 0 : ((uint64_t)a >> sh);
      pb = sh >= 32 ? 0 : ((uint64_t)b >> sh);
      used = used + width - 64;
    } else {
      used += width;
    }
  }
  __device__ __forceinline__ void lin(const WarpCtx& c, uint32_t v) { push(c, v, v, 0xFFFFFFFFu, 32); }
  __device__ __forceinline__ uint32_t add(const WarpCtx& c, uint32_t x, uint32_t y) {
    uint32_t sum = x + y;
    uint32_t cin = sum ^ x ^ y;
    uint32_t l = (x ^ cin) & 0x7FFFFFFFu, r = (y ^ cin) & 0x7FFFFFFFu;
    push(c, l & r, l, r, 31);
    return sum;
  }
};

#define WG(LA, LB, LC, LD, R, S)                                        \
  {                                                                     \
    uint32_t a_ = s[LA], b_ = s[LB], c_ = s[LC], d_ = s[LD];            \
    uint32_t mx = mp[S], my = mp[S + 1];                                \
    uint32_t t0 = k.add(c, a_, b_);                                     \
    uint32_t a1 = k.add(c, t0, mx);                                     \
    uint32_t d1 = b3::rotr(d_ ^ a1, 16);                                \
    uint32_t c1 = k.add(c, c_, d1);                                     \
    uint32_t b1 = b3::rotr(b_ ^ c1, 12);                                \
    uint32_t t1 = k.add(c, a1, b1);                                     \
    uint32_t a2 = k.add(c, t1, my);                                     \
    uint32_t d2 = b3::rotr(d1 ^ a2, 8);                                 \
    uint32_t c2 = k.add(c, c1, d2);                                     \
    uint32_t bn = b3::rotr(b1 ^ c2, 7);                                 \
    k.lin(c, bn);                                                       \
    k.lin(c, d2);                                                       \
    s[LA] = a2; s[LB] = bn; s[LC] = c2; s[LD] = d2;                     \
  }

__global__ void __launch_bounds__(32 * WARPS_PER_BLOCK)
witness_kernel(const flock_compression* __restrict__ in, size_t n_in, size_t n_total, uint64_t* gz,
               uint64_t* ga, uint64_t* gb, uint8_t* stripe) {
  extern __shared__ uint64_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t slot = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t warp_slot0 = slot - lane;
  if (warp_slot0 >= n_total) return;
  WarpCtx c;
  uint64_t* base = smem + (size_t)warp * 3 * 32 * STAGE_STRIDE;
  c.sz = base;
  c.sa = base + 32 * STAGE_STRIDE;
  c.sb = base + 64 * STAGE_STRIDE;
  c.gz = gz; c.ga = ga; c.gb = gb; c.stripe = stripe;
  c.warp_slot0 = warp_slot0;
  size_t rem = n_total - warp_slot0;
  c.n_valid = rem >= 32 ? 32 : (int)rem;
  c.lane = lane;

  // Inputs: real compression, or the all-zero padding compression.
  uint32_t cv[8], m[16];
  uint64_t counter = 0;
  uint32_t blen = 0, flg = 0;
  if (slot < n_in) {
    const flock_compression& x = in[slot];
#pragma unroll
    for (int i = 0; i < 8; i++) cv[i] = x.cv[i];
#pragma unroll
    for (int i = 0; i < 16; i++) m[i] = x.m[i];
    counter = x.counter; blen = x.block_len; flg = x.flags;
  } else {
#pragma unroll
    for (int i = 0; i < 8; i++) cv[i] = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) m[i] = 0;
  }
  // out_lo sits before the G blocks in the layout: compute the output first.
  uint32_t out[16];
  b3::compress(cv, m, counter, blen, flg, out);

  Sink k{0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 8; i++) k.lin(c, cv[i]);
#pragma unroll
  for (int i = 0; i < 8; i++) k.lin(c, out[i]);
  k.push(c, 1, 1, 1, 1);  // constant wire at bit 512
#pragma unroll
  for (int i = 0; i < 16; i++) k.lin(c, m[i]);
  uint32_t tlo = (uint32_t)counter, thi = (uint32_t)(counter >> 32);
  k.lin(c, tlo);
  k.lin(c, thi);
  k.lin(c, blen);
  k.lin(c, flg);
  uint32_t s[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    b3::IV(0), b3::IV(1), b3::IV(2), b3::IV(3), tlo, thi, blen, flg};
  uint32_t mp[16];  // this round's message order
#pragma unroll
  for (int i = 0; i < 16; i++) mp[i] = m[i];
#pragma unroll
  for (int r = 0; r < 7; r++) {
    WG(0, 4, 8, 12, r, 0);
    WG(1, 5, 9, 13, r, 2);
    WG(2, 6, 10, 14, r, 4);
    WG(3, 7, 11, 15, r, 6);
    WG(0, 5, 10, 15, r, 8);
    WG(1, 6, 11, 12, r, 10);
    WG(2, 7, 8, 13, r, 12);
    WG(3, 4, 9, 14, r, 14);
    if (r < 6) b3::permute(mp);
  }
#pragma unroll
  for (int i = 0; i < 8; i++) k.lin(c, s[i + 8] ^ cv[i]);  // out_hi
  // Flush the partial word, then zero words up to the end of the block.
  k.emit(c, k.pz, k.pa, k.pb);
  while (k.word < KWORDS) k.emit(c, 0, 0, 0);
}

}  // namespace

int flock_launch_witness(const flock_compression* d_in, size_t n_in, int n_blocks_log, void* d_z, void* d_a,
                         void* d_b, void* d_stripe, cudaStream_t stream) {
  size_t n_total = (size_t)1 << n_blocks_log;
  if (n_in > n_total || n_blocks_log < 3) return FLOCK_ERR_SHAPE;
  if ((d_a == nullptr) != (d_b == nullptr)) return FLOCK_ERR_SHAPE;
  const int threads = 32 * WARPS_PER_BLOCK;
  size_t blocks = (n_total + threads - 1) / threads;
  size_t smem = (size_t)WARPS_PER_BLOCK * 3 * 32 * STAGE_STRIDE * sizeof(uint64_t);
  flock_once_per_device((const void*)witness_kernel, [] {
    cudaFuncSetAttribute(witness_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(WARPS_PER_BLOCK * 3 * 32 * STAGE_STRIDE * sizeof(uint64_t)));
  });
  witness_kernel<<<(unsigned)blocks, threads, smem, stream>>>(d_in, n_in, n_total, (uint64_t*)d_z,
                                                              (uint64_t*)d_a, (uint64_t*)d_b, (uint8_t*)d_stripe); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

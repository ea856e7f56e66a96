// Hash-chain relation kernels: the per-instance region fold of the committed
// witness (crates/flock-prover/src/r1cs_hashes/chain_common.rs:124-176), the
// shift sumcheck over (instance, selector) tables (crates/flock-prover/src/chain.rs:155-233)
// and the packed-direct claim's eq tensor added to the combined PCS basis
// (crates/flock-core/src/pcs.rs:1055-1090).
//
// BLAKE3 layout (r1cs_hashes/blake3.rs:3750-3757): each instance is a block of
// 2^14 witness bits = 128 packed F128 words; its input cv is words 0, 1 and
// its output cv words 2, 3. The sumcheck tables hold 2^(n+1) entries indexed
// by y + 2^n s0, and every round binds the top remaining variable.
#include "flock_internal.h"
#include "gf128.cuh"

namespace {

constexpr int CH_THREADS = 256;
constexpr size_t kWordsPerBlock = 128;

inline gf128 to_gf(const uint64_t v[2]) {
  gf128 r;
  r.w[0] = (uint32_t)v[0]; r.w[1] = (uint32_t)(v[0] >> 32); r.w[2] = (uint32_t)v[1]; r.w[3] = (uint32_t)(v[1] >> 32);
  return r;
}
inline unsigned grid_for(size_t work, size_t threads, size_t cap) {
  size_t g = (work + threads - 1) / threads;
  if (g < 1) g = 1;
  return (unsigned)(g > cap ? cap : g);
}

// g[i] = e0 z[128 i] + e1 z[128 i + 1]; g[n + i] = e0 z[128 i + 2] + e1 z[128 i + 3].
__global__ void chain_fold_io_kernel(const uint4* __restrict__ z, size_t n, gf128 e0, gf128 e1,
                                     gf128* __restrict__ g) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint4* w = z + i * kWordsPerBlock;
    uint4 v0 = __ldg(w), v1 = __ldg(w + 1), v2 = __ldg(w + 2), v3 = __ldg(w + 3);
    gf128 a0 = {{v0.x, v0.y, v0.z, v0.w}}, a1 = {{v1.x, v1.y, v1.z, v1.w}};
    gf128 b0 = {{v2.x, v2.y, v2.z, v2.w}}, b1 = {{v3.x, v3.y, v3.z, v3.w}};
    g[i] = gf_add(gf_mul(e0, a0), gf_mul(e1, a1));
    g[n + i] = gf_add(gf_mul(e0, b0), gf_mul(e1, b1));
  }
}

// W[y] = eq(tau, y - 1) for y >= 1, W[0] = alpha, W[n + y] = eq(tau, y);
// eq(tau, y) = lo[y & mask] * hi[y >> lo_bits].
__global__ void chain_weights_kernel(const gf128* __restrict__ lo, const gf128* __restrict__ hi, int lo_bits, size_t n,
                                     gf128 alpha, gf128* __restrict__ W) {
  const size_t mask = ((size_t)1 << lo_bits) - 1;
  for (size_t y = (size_t)blockIdx.x * blockDim.x + threadIdx.x; y < n; y += (size_t)gridDim.x * blockDim.x) {
    gf128 e = gf_mul(lo[y & mask], hi[y >> lo_bits]);
    W[n + y] = e;
    if (y + 1 < n) W[y + 1] = e;
    if (y == 0) W[0] = alpha;
  }
}

// With bind: the 2h-entry tables W, g are bound at r in their top variable
// (x' = x_lo + r (x_hi + x_lo)) into their first h entries, in place (thread i
// owns entries i, i + h/2, i + h, i + 3h/2). Then the round message over the
// h-entry tables: q(1) = sum W_hi g_hi, q(inf) = sum (W_lo + W_hi)(g_lo + g_hi),
// halves split at h/2; per-block partials (q(1), q(inf)).
__global__ void __launch_bounds__(CH_THREADS)
chain_round_kernel(gf128* __restrict__ W, gf128* __restrict__ g, size_t h, int bind, const __grid_constant__ gf128p r,
                   gf128* __restrict__ partials) {
  const size_t q = h / 2;
  gf256 e1 = {{0, 0, 0, 0}}, ei = e1;
  for (size_t i = (size_t)blockIdx.x * CH_THREADS + threadIdx.x; i < q; i += (size_t)gridDim.x * CH_THREADS) {
    gf128 wl = W[i], wh = W[i + q], gl = g[i], gh = g[i + q];
    if (bind) {
      wl = gf_add(wl, gf_mul_p(gf_add(W[i + h], wl), r));
      wh = gf_add(wh, gf_mul_p(gf_add(W[i + q + h], wh), r));
      gl = gf_add(gl, gf_mul_p(gf_add(g[i + h], gl), r));
      gh = gf_add(gh, gf_mul_p(gf_add(g[i + q + h], gh), r));
      W[i] = wl; W[i + q] = wh; g[i] = gl; g[i + q] = gh;
    }
    gf256_acc(e1, gf_mul_wide(wh, gh));
    gf256_acc(ei, gf_mul_wide(gf_add(wl, wh), gf_add(gl, gh)));
  }
  __shared__ gf256 red[2][CH_THREADS / 32];
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      e1.r[k] ^= __shfl_xor_sync(0xffffffffu, e1.r[k], off);
      ei.r[k] ^= __shfl_xor_sync(0xffffffffu, ei.r[k], off);
    }
  const int wp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][wp] = e1; red[1][wp] = ei; }
  __syncthreads();
  if (threadIdx.x == 0) {
    gf256 s1 = {{0, 0, 0, 0}}, si = s1;
    for (int k = 0; k < CH_THREADS / 32; k++) { gf256_acc(s1, red[0][k]); gf256_acc(si, red[1][k]); }
    partials[2 * blockIdx.x] = gf256_reduce(s1);
    partials[2 * blockIdx.x + 1] = gf256_reduce(si);
  }
}

struct Coef4 { gf128 c[4]; };

// The packed-direct claim's eq tensor, scaled by its batching challenge:
// b[128 i + p] += c[p] eq(instance_point, i) for p < 4. The claim point's
// five zero coordinates (selector bits above the in/out bit) leave every
// other word of a block untouched.
__global__ void chain_claim_basis_kernel(gf128* __restrict__ b, size_t n, const gf128* __restrict__ lo,
                                         const gf128* __restrict__ hi, int lo_bits, Coef4 c) {
  const size_t mask = ((size_t)1 << lo_bits) - 1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    gf128 e = gf_mul(lo[i & mask], hi[i >> lo_bits]);
    gf128* w = b + i * kWordsPerBlock;
#pragma unroll
    for (int p = 0; p < 4; p++) w[p] = gf_add(w[p], gf_mul(c.c[p], e));
  }
}

}  // namespace

int flock_launch_chain_fold_io(const void* z, size_t n_inst, const uint64_t e0[2], const uint64_t e1[2], void* g,
                               cudaStream_t st) {
  chain_fold_io_kernel<<<grid_for(n_inst, CH_THREADS, 152 * 8), CH_THREADS, 0, st>>>(
      (const uint4*)z, n_inst, to_gf(e0), to_gf(e1), (gf128*)g);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_chain_weights(const void* lo, const void* hi, int lo_bits, size_t n_inst, const uint64_t alpha[2],
                               void* W, cudaStream_t st) {
  chain_weights_kernel<<<grid_for(n_inst, CH_THREADS, 152 * 8), CH_THREADS, 0, st>>>(
      (const gf128*)lo, (const gf128*)hi, lo_bits, n_inst, to_gf(alpha), (gf128*)W);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_chain_round_grid(size_t h) { return (int)grid_for(h / 2, CH_THREADS, 152 * 4); }

int flock_launch_chain_round(void* W, void* g, size_t h, int bind, const uint64_t r[2], void* partials, int grid,
                             cudaStream_t st) {
  if (h < 2) return FLOCK_ERR_SHAPE;
  chain_round_kernel<<<grid, CH_THREADS, 0, st>>>((gf128*)W, (gf128*)g, h, bind, gf_prepare(to_gf(r)),
                                                  (gf128*)partials);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_chain_claim_basis(void* b, size_t n_inst, const void* lo, const void* hi, int lo_bits,
                                   const uint64_t c[8], cudaStream_t st) {
  Coef4 k;
  for (int p = 0; p < 4; p++) k.c[p] = to_gf(c + 2 * p);
  chain_claim_basis_kernel<<<grid_for(n_inst, CH_THREADS, 152 * 8), CH_THREADS, 0, st>>>(
      (gf128*)b, n_inst, (const gf128*)lo, (const gf128*)hi, lo_bits, k);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

// Lincheck kernels (crates/flock-core/src/lincheck.rs:1480-1660).
//
//  * partial fold: z_vec[i] = sum_outer z[i, outer] eq(x_outer, outer), read
//    from the byte stripe (byte (outer/8)*2^14 + i holds 8 outer bits), one
//    256-entry subset-sum table of eq per stripe, eight stripes per round
//    (lincheck.rs:655-720);
//  * comb: alpha * A0^T eq_inner + B0^T eq_inner (+ beta at the constant
//    column) gathered column-wise from a CSC copy of the base matrices;
//  (the product sumcheck rounds over (comb, z_vec), binding the top variable
//  (lincheck.rs:1242-1300), run on flock_launch_chain_round).
#include "flock_internal.h"
#include "gf128.cuh"

namespace {

constexpr int PF_THREADS = 256;
constexpr int PF_PER_THREAD = 16;                                    // bytes (columns) per thread
constexpr int PF_SLICES = FLOCK_K / (PF_THREADS * PF_PER_THREAD);  // column slices: 4

constexpr int PF_GROUP = 8;  // stripes per table round (64 outer indices)

// CTA (slice, part): columns [slice * 4096, +4096) of the stripe groups
// part, part + parts, ... Per round: 64 eq weights (one product each, 64
// threads), PF_GROUP subset-sum tables of 256 entries, then every thread folds
// its 16 bytes of each stripe. Grouping amortises the barriers and the table
// build over eight stripes; the four column slices keep 64 accumulator
// registers per thread affordable.
__global__ void __launch_bounds__(PF_THREADS, 2)
lc_partial_fold_kernel(const uint8_t* __restrict__ stripe, size_t n_stripes, const gf128* __restrict__ eq_lo,
                       const gf128* __restrict__ eq_hi, int lo_bits, gf128* __restrict__ partials) {
  // t8[v][q]: subset sums of stripe q's eight eq weights; entry (v, q) sits in
  // bank group q, and lane l starts at stripe l mod 8, so eight consecutive
  // lanes read eight distinct bank groups. e8v[r][q]: weight of bit r of stripe q.
  __shared__ gf128 t8[256][PF_GROUP];
  __shared__ gf128 e8v[8][PF_GROUP];
  const int lane8 = threadIdx.x & 7;
  gf128 acc[PF_PER_THREAD];
#pragma unroll
  for (int k = 0; k < PF_PER_THREAD; k++) acc[k] = gf_zero();
  const int slice = blockIdx.x % PF_SLICES;
  const size_t part = blockIdx.x / PF_SLICES, parts = gridDim.x / PF_SLICES;
  const size_t col0 = (size_t)slice * PF_THREADS * PF_PER_THREAD + (size_t)threadIdx.x * PF_PER_THREAD;
  const size_t lo_mask = ((size_t)1 << lo_bits) - 1;
  const size_t n_groups = n_stripes / PF_GROUP;
  for (size_t g = part; g < n_groups; g += parts) {
    const size_t s0 = g * PF_GROUP;
    if (threadIdx.x < PF_GROUP * 8) {
      size_t o = 8 * s0 + threadIdx.x;  // stripe threadIdx.x / 8, bit threadIdx.x % 8
      e8v[threadIdx.x & 7][threadIdx.x >> 3] = gf_mul(eq_lo[o & lo_mask], eq_hi[o >> lo_bits]);
    }
    // this thread's bytes of the group's stripes (loads overlap the table build)
    uint4 bytes[PF_GROUP];
#pragma unroll
    for (int q = 0; q < PF_GROUP; q++)
      bytes[q] = *reinterpret_cast<const uint4*>(stripe + (s0 + q) * FLOCK_K + col0);
    __syncthreads();
    // subset sums by a Gray walk: thread (c, q) owns t8[8c .. 8c+7][q], starts
    // from the sum over the bits of 8c and adds one weight per entry
    static_assert(PF_THREADS == 32 * PF_GROUP, "one thread per (8-entry run, stripe)");
    {
      const int q = threadIdx.x & 7, c = threadIdx.x >> 3;
      gf128 acc8 = gf_zero();
#pragma unroll
      for (int r = 3; r < 8; r++)
        if ((c >> (r - 3)) & 1) acc8 = gf_add(acc8, e8v[r][q]);
#pragma unroll
      for (int i = 0; i < 8; i++) {
        if (i) acc8 = gf_add(acc8, e8v[(i & 1) ? 0 : (i & 2) ? 1 : 2][q]);
        t8[8 * c + (i ^ (i >> 1))][q] = acc8;
      }
    }
    __syncthreads();
#pragma unroll
    for (int st = 0; st < PF_GROUP; st++) {
      const int q = (lane8 + st) & (PF_GROUP - 1);  // rotated stripe
      uint4 bq = bytes[0];
#pragma unroll
      for (int qq = 1; qq < PF_GROUP; qq++)
        if (q == qq) bq = bytes[qq];
      const uint32_t wds[4] = {bq.x, bq.y, bq.z, bq.w};
#pragma unroll
      for (int k = 0; k < PF_PER_THREAD; k++) {
        uint32_t b = (wds[k >> 2] >> (8 * (k & 3))) & 255;
        if (b) acc[k] = gf_add(acc[k], t8[b][q]);
      }
    }
    __syncthreads();
  }
  gf128* out = partials + part * FLOCK_K + col0;
#pragma unroll
  for (int k = 0; k < PF_PER_THREAD; k++) out[k] = acc[k];
}

// comb[c] = alpha * sum_{r in colA(c)} eq[r] + sum_{r in colB(c)} eq[r] (+ beta at pin).
// One warp per column: the lanes stride over the column's row indices
// (coalesced index reads, independent gathers of eq from L2) and XOR-reduce;
// columns hold 0..7.4 K entries (930 + 355 on average).
constexpr int LC_COMB_THREADS = 256;
__global__ void __launch_bounds__(LC_COMB_THREADS)
lc_comb_kernel(const uint32_t* __restrict__ a_ptr, const uint32_t* __restrict__ a_idx,
               const uint32_t* __restrict__ b_ptr, const uint32_t* __restrict__ b_idx,
               const gf128* __restrict__ eq, gf128 alpha, gf128 beta, int pin, gf128* __restrict__ comb) {
  const int c = (int)((blockIdx.x * (size_t)LC_COMB_THREADS + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (c >= FLOCK_K) return;
  gf128 sa = gf_zero(), sb = gf_zero();
  for (uint32_t k = a_ptr[c] + lane, e = a_ptr[c + 1]; k < e; k += 32) sa = gf_add(sa, eq[a_idx[k]]);
  for (uint32_t k = b_ptr[c] + lane, e = b_ptr[c + 1]; k < e; k += 32) sb = gf_add(sb, eq[b_idx[k]]);
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      sa.w[q] ^= __shfl_xor_sync(0xffffffffu, sa.w[q], off);
      sb.w[q] ^= __shfl_xor_sync(0xffffffffu, sb.w[q], off);
    }
  if (lane == 0) {
    gf128 v = gf_add(gf_mul(alpha, sa), sb);
    if (c == pin) v = gf_add(v, beta);
    comb[c] = v;
  }
}

// Quirky eq table (lincheck.rs:1127-1143): out[s + 64 * j] = lag[s] * eq(x_inner_rest)[j].
__global__ void lc_quirky_eq_kernel(const gf128* __restrict__ lag, const gf128* __restrict__ x_rest, int n_rest,
                                    gf128* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (64 << n_rest)) return;
  int s = i & 63, j = i >> 6;
  gf128 e = gf_one();
  for (int k = 0; k < n_rest; k++) {
    gf128 r = x_rest[k];
    if (!((j >> k) & 1)) r.w[0] ^= 1;
    e = gf_mul(e, r);
  }
  out[i] = gf_mul(lag[s], e);
}

inline gf128 to_gf(const uint64_t v[2]) {
  gf128 r;
  r.w[0] = (uint32_t)v[0]; r.w[1] = (uint32_t)(v[0] >> 32); r.w[2] = (uint32_t)v[1]; r.w[3] = (uint32_t)(v[1] >> 32);
  return r;
}

}  // namespace

// grid = number of partial rows (stripe-group partitions); partials: grid x 2^14.
int flock_launch_lc_partial_fold(const void* stripe, size_t n_stripes, const void* eq_lo, const void* eq_hi,
                                 int lo_bits, void* partials, int grid, cudaStream_t st) {
  if (n_stripes % PF_GROUP != 0) return FLOCK_ERR_SHAPE;
  lc_partial_fold_kernel<<<grid * PF_SLICES, PF_THREADS, 0, st>>>((const uint8_t*)stripe, n_stripes,
                                                                  (const gf128*)eq_lo, (const gf128*)eq_hi, lo_bits,
                                                                  (gf128*)partials);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_lc_comb(const uint32_t* a_ptr, const uint32_t* a_idx, const uint32_t* b_ptr, const uint32_t* b_idx,
                         const void* eq, const uint64_t alpha[2], const uint64_t beta[2], int pin, void* comb,
                         cudaStream_t st) {
  lc_comb_kernel<<<FLOCK_K * 32 / LC_COMB_THREADS, LC_COMB_THREADS, 0, st>>>(a_ptr, a_idx, b_ptr, b_idx,
                                                                            (const gf128*)eq, to_gf(alpha),
                                                to_gf(beta), pin, (gf128*)comb); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_lc_quirky_eq(const void* lag, const void* x_rest, int n_rest, void* out, cudaStream_t st) {
  int n = 64 << n_rest;
  lc_quirky_eq_kernel<<<(n + 255) / 256, 256, 0, st>>>((const gf128*)lag, (const gf128*)x_rest, n_rest,
                                                       (gf128*)out); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}


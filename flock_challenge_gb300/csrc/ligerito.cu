// Ligerito PCS prover kernels (crates/flock-core/src/pcs/ligerito.rs).
//
//  * round message (ligerito.rs:3725-3773): u0 = sum f0 b0, u2 = sum (f0+f1)(b0+b1)
//    over LSB pairs, fused with the preceding fold f' = f0 + r (f0 + f1)
//    (ligerito.rs:5517-5566, partial_eval_lsb :1673-1691);
//  * OOD introduction with b_new = eq(z) evaluated on the fly from split
//    tables, returning the message and h = sum f eq (ligerito.rs:5684-5702),
//    and its glue b += beta eq(z);
//  * induced basis (ligerito.rs:1989-2160): basis[j] = sum_i alpha_i Xhat_j(q_i)
//    with Xhat_j = prod_{k in bits(j)} What_k; computed as a sum over queries of
//    products of low/high tensor halves;
//  * glue b += beta * basis, row and tree-node gathers for openings.
#include "flock_internal.h"
#include "gf128.cuh"
#include "gf_tab.cuh"

namespace {

constexpr int LG_THREADS = 256;
#ifndef LG_MIN_BLOCKS
#define LG_MIN_BLOCKS 2  // resident blocks per SM of the fold/message kernels
#endif

__device__ __forceinline__ void block_reduce_write(gf256 a, gf256 b, gf256 c, gf128* out) {
  __shared__ gf256 red[3][LG_THREADS / 32];
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      a.r[k] ^= __shfl_xor_sync(0xffffffffu, a.r[k], off);
      b.r[k] ^= __shfl_xor_sync(0xffffffffu, b.r[k], off);
      c.r[k] ^= __shfl_xor_sync(0xffffffffu, c.r[k], off);
    }
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = a; red[1][w] = b; red[2][w] = c; }
  __syncthreads();
  if (threadIdx.x == 0) {
    gf256 s0 = {{0, 0, 0, 0}}, s1 = s0, s2 = s0;
    for (int k = 0; k < LG_THREADS / 32; k++) { gf256_acc(s0, red[0][k]); gf256_acc(s1, red[1][k]); gf256_acc(s2, red[2][k]); }
    out[3 * blockIdx.x] = gf256_reduce(s0);
    out[3 * blockIdx.x + 1] = gf256_reduce(s1);
    out[3 * blockIdx.x + 2] = gf256_reduce(s2);
  }
}

// If fold: in has 2 * n_out elements, bound at r into out (n_out elements);
// message over the n_out-element state. Partials: (u0, u2, 0) per block.
// use_tab: the fold multiplies through r's byte tables (gf_tab.cuh, dynamic
// shared memory), worth their build when a CTA folds hundreds of pairs.
__global__ void __launch_bounds__(LG_THREADS, LG_MIN_BLOCKS)
lig_fold_msg_kernel(const gf128* __restrict__ f, const gf128* __restrict__ b, size_t n_out, int fold,
                    const __grid_constant__ gf128p r, const gf128 r_plain, int use_tab,
                    gf128* __restrict__ fo, gf128* __restrict__ bo, gf128* __restrict__ partials) {
  extern __shared__ uint4 rtab[];
  const uint32_t rot = threadIdx.x & 15;
  if (use_tab) gf_tab_build(r_plain, rtab);
  gf256 u0 = {{0, 0, 0, 0}}, u2 = u0, zz = u0;
  size_t pairs = n_out / 2;
  for (size_t j = (size_t)blockIdx.x * LG_THREADS + threadIdx.x; j < pairs; j += (size_t)gridDim.x * LG_THREADS) {
    gf128 f0, f1, b0, b1;
    if (fold) {
      gf128 x0 = f[4 * j], x1 = f[4 * j + 1], x2 = f[4 * j + 2], x3 = f[4 * j + 3];
      gf128 y0 = b[4 * j], y1 = b[4 * j + 1], y2 = b[4 * j + 2], y3 = b[4 * j + 3];
      if (use_tab) {
        f0 = gf_add(x0, gf_mul_tab(rtab, gf_add(x0, x1), rot));
        f1 = gf_add(x2, gf_mul_tab(rtab, gf_add(x2, x3), rot));
        b0 = gf_add(y0, gf_mul_tab(rtab, gf_add(y0, y1), rot));
        b1 = gf_add(y2, gf_mul_tab(rtab, gf_add(y2, y3), rot));
      } else {
        f0 = gf_add(x0, gf_mul_p(gf_add(x0, x1), r));
        f1 = gf_add(x2, gf_mul_p(gf_add(x2, x3), r));
        b0 = gf_add(y0, gf_mul_p(gf_add(y0, y1), r));
        b1 = gf_add(y2, gf_mul_p(gf_add(y2, y3), r));
      }
      fo[2 * j] = f0; fo[2 * j + 1] = f1;
      bo[2 * j] = b0; bo[2 * j + 1] = b1;
    } else {
      f0 = f[2 * j]; f1 = f[2 * j + 1]; b0 = b[2 * j]; b1 = b[2 * j + 1];
    }
    gf256_acc(u0, gf_mul_wide(f0, b0));
    gf256_acc(u2, gf_mul_wide(gf_add(f0, f1), gf_add(b0, b1)));
  }
  block_reduce_write(u0, u2, zz, partials);
}

// Message of (f, eq(z)) and h = sum f * eq(z); eq(z)[j] = lo[j & mask] * hi[j >> lo_bits].
__global__ void __launch_bounds__(LG_THREADS, 2)
lig_intro_eq_kernel(const gf128* __restrict__ f, size_t n, const gf128* __restrict__ lo,
                    const gf128* __restrict__ hi, int lo_bits, gf128* __restrict__ partials) {
  gf256 u0 = {{0, 0, 0, 0}}, u2 = u0, h = u0;
  size_t mask = ((size_t)1 << lo_bits) - 1;
  for (size_t j = (size_t)blockIdx.x * LG_THREADS + threadIdx.x; j < n / 2; j += (size_t)gridDim.x * LG_THREADS) {
    size_t i0 = 2 * j, i1 = 2 * j + 1;
    gf128 e0 = gf_mul(lo[i0 & mask], hi[i0 >> lo_bits]);
    gf128 e1 = gf_mul(lo[i1 & mask], hi[i1 >> lo_bits]);
    gf128 f0 = f[i0], f1 = f[i1];
    gf256 p0 = gf_mul_wide(f0, e0);
    gf256_acc(u0, p0);
    gf256_acc(h, p0);
    gf256_acc(h, gf_mul_wide(f1, e1));
    gf256_acc(u2, gf_mul_wide(gf_add(f0, f1), gf_add(e0, e1)));
  }
  block_reduce_write(u0, u2, h, partials);
}

__global__ void glue_eq_kernel(gf128* __restrict__ b, size_t n, const gf128* __restrict__ lo,
                               const gf128* __restrict__ hi, int lo_bits, gf128 beta) {
  size_t mask = ((size_t)1 << lo_bits) - 1;
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    b[j] = gf_add(b[j], gf_mul(beta, gf_mul(lo[j & mask], hi[j >> lo_bits])));
}

__global__ void glue_kernel(gf128* __restrict__ b, const gf128* __restrict__ add, size_t n, gf128 beta) {
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    b[j] = gf_add(b[j], gf_mul(beta, add[j]));
}

// What_k(q_i) for k < n (ligerito.rs:1776-1824: s_0 = q, s_k = s^2 + s_{k-1}(v_{k-1}) s,
// normalized by 1 / s_k(v_k)). Each s_k is GF(2)-linear in its argument (a
// square plus a constant multiple of a linear map), so What_k(q) is the XOR,
// over the set bits b of the 32-bit index q, of lin[k][b] = What_k(x^b): one
// thread per (query, k), no product.
__global__ void what_kernel(const uint32_t* __restrict__ queries, int nq, int n, const gf128* __restrict__ lin,
                            gf128* __restrict__ W) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)nq * n) return;
  const int i = (int)(e / n), k = (int)(e % n);
  const uint32_t q = queries[i];
  const gf128* row = lin + (size_t)k * 32;
  gf128 acc = gf_zero();
  for (int b = 0; b < 32; b++)
    if ((q >> b) & 1) acc = gf_add(acc, row[b]);
  W[e] = acc;
}

// T[i][j] = scale_i * prod_{k < bits, bit k of j} W[i][k0 + k]; scale_i = alpha_i or 1.
// CTA (query i, chunk c) first builds the sub-tables of the low TB_LO bits
// (scaled) and of the remaining high bits (at most TB_HI) in shared memory,
// then forms its 256 entries with one product each (a chain of up to `bits`
// dependent products per entry before).
constexpr int TB_LO = 5, TB_HI = 7, TB_THREADS = 256;
static_assert((1 << TB_LO) <= 32 && 32 + (1 << TB_HI) <= TB_THREADS, "sub-table builders fit the CTA");
__global__ void __launch_bounds__(TB_THREADS)
tensor_kernel(const gf128* __restrict__ W, int nq, int n, int k0, int bits, const gf128* __restrict__ scale,
              gf128* __restrict__ T) {
  __shared__ gf128 lo_t[1 << TB_LO], hi_t[1 << TB_HI];
  const int lb = bits < TB_LO ? bits : TB_LO, hb = bits - lb;
  const size_t len = (size_t)1 << bits;
  const size_t chunks = (len + TB_THREADS - 1) / TB_THREADS;
  const int i = (int)(blockIdx.x / chunks);
  const size_t c = blockIdx.x % chunks;
  const gf128* w = W + (size_t)i * n + k0;
  const int t = threadIdx.x;
  if (t < (1 << lb)) {
    gf128 acc = scale ? scale[i] : gf_one();
    for (int k = 0; k < lb; k++)
      if ((t >> k) & 1) acc = gf_mul(acc, w[k]);
    lo_t[t] = acc;
  } else if (t >= 32 && t - 32 < (1 << hb)) {
    const int u = t - 32;
    gf128 acc = gf_one();
    for (int k = 0; k < hb; k++)
      if ((u >> k) & 1) acc = gf_mul(acc, w[lb + k]);
    hi_t[u] = acc;
  }
  __syncthreads();
  const size_t j = c * TB_THREADS + t;
  if (j < len) T[(size_t)i * len + j] = gf_mul(lo_t[j & ((1 << lb) - 1)], hi_t[j >> lb]);
}

// basis[j] = sum_i LO[i][j & mask] * HI[i][j >> lo_bits]. Slice blockIdx.y
// sums the queries [y q_per, (y + 1) q_per) into row y of out (the slices'
// rows are then XOR-reduced), so small bases still fill the GPU.
__global__ void __launch_bounds__(256)
basis_kernel(const gf128* __restrict__ LO, const gf128* __restrict__ HI, int nq, int lo_bits, int hi_bits,
             int q_per, gf128* __restrict__ out) {
  size_t n = (size_t)1 << (lo_bits + hi_bits);
  size_t lo_n = (size_t)1 << lo_bits, hi_n = (size_t)1 << hi_bits;
  const int i0 = blockIdx.y * q_per, i1 = i0 + q_per < nq ? i0 + q_per : nq;
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    size_t jl = j & (lo_n - 1), jh = j >> lo_bits;
    gf256 acc = {{0, 0, 0, 0}};
    for (int i = i0; i < i1; i++) gf256_acc(acc, gf_mul_wide(LO[(size_t)i * lo_n + jl], HI[(size_t)i * hi_n + jh]));
    out[(size_t)blockIdx.y * n + j] = gf256_reduce(acc);
  }
}

// The same basis through byte tables, for large bases (LO_BITS = 10 or 11):
// CTA h owns the 2^LO_BITS entries of high index h and walks the queries; per
// query it builds the byte tables of HI[i][h] (one row per thread, computed
// directly) and adds HI[i][h] LO[i][jl] for its entries (four or eight per
// thread) as 16 table lookups each instead of a carry-less multiply. A barrier
// before each build orders the previous query's lookups before the new
// writes, so one table suffices; three CTAs per SM overlap one CTA's build
// with the others' lookups.
constexpr int BT_THREADS = 256;
constexpr size_t BT_SMEM = (size_t)GF_TAB_ENTRIES * 16;
static_assert(BT_THREADS == 256, "one byte-table row per thread");

template <int LO_BITS>
__global__ void __launch_bounds__(BT_THREADS, 3)
basis_tab_kernel(const gf128* __restrict__ LO, const gf128* __restrict__ HI, int nq, int hi_bits,
                 gf128* __restrict__ basis) {
  constexpr int PER_THREAD = (1 << LO_BITS) / BT_THREADS;
  extern __shared__ uint4 btab[];
  const size_t lo_n = (size_t)1 << LO_BITS, hi_n = (size_t)1 << hi_bits;
  const uint32_t rot = threadIdx.x & 7;
  for (size_t h = blockIdx.x; h < hi_n; h += gridDim.x) {
    gf128 acc[PER_THREAD];
#pragma unroll
    for (int k = 0; k < PER_THREAD; k++) acc[k] = gf_zero();
    for (int i = 0; i < nq; i++) {
      __syncthreads();
      gf_tab_row_direct(HI[(size_t)i * hi_n + h], btab, threadIdx.x);
      __syncthreads();
      const gf128* lo = LO + (size_t)i * lo_n + threadIdx.x;
#pragma unroll
      for (int k = 0; k < PER_THREAD; k++) acc[k] = gf_add(acc[k], gf_mul_tab(btab, lo[k * BT_THREADS], rot));
    }
    gf128* out = basis + (h << LO_BITS) + threadIdx.x;
#pragma unroll
    for (int k = 0; k < PER_THREAD; k++) out[k * BT_THREADS] = acc[k];
  }
}

// out[j] = in[2j] + r (in[2j] + in[2j+1]): one LSB fold (ligerito.rs:1673-1691).
__global__ void fold_lsb_kernel(const gf128* __restrict__ in, size_t n_out, const __grid_constant__ gf128p r,
                                gf128* __restrict__ out) {
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_out; j += (size_t)gridDim.x * blockDim.x) {
    const gf128 x0 = in[2 * j], x1 = in[2 * j + 1];
    out[j] = gf_add(x0, gf_mul_p(gf_add(x0, x1), r));
  }
}

__global__ void gather_rows_kernel(const gf128* __restrict__ mat, const uint32_t* __restrict__ rows, int n_rows,
                                   int width, gf128* __restrict__ out) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n_rows * width) return;
  size_t r = e / width, c = e % width;
  out[e] = mat[(size_t)rows[r] * width + c];
}

__global__ void gather_nodes_kernel(const uint4* __restrict__ tree, const uint32_t* __restrict__ idx, int n,
                                    uint4* __restrict__ out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 2 * n) return;
  out[e] = tree[2 * (size_t)idx[e >> 1] + (e & 1)];
}

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

}  // namespace

int flock_lig_grid(size_t n_pairs) { return (int)grid_for(n_pairs, LG_THREADS, 152 * 4); }

int flock_launch_lig_fold_msg(const void* f, const void* b, size_t n_out, int fold, const uint64_t r[2], void* fo,
                              void* bo, void* partials, int grid, cudaStream_t st) {
  constexpr size_t kTabSmem = (size_t)GF_TAB_ENTRIES * 16;
  flock_once_per_device((const void*)lig_fold_msg_kernel, [] {
    cudaFuncSetAttribute(lig_fold_msg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTabSmem);
  });
  const int use_tab = fold && (n_out / 2) / (size_t)grid >= 512;
  lig_fold_msg_kernel<<<grid, LG_THREADS, use_tab ? kTabSmem : 0, st>>>(
      (const gf128*)f, (const gf128*)b, n_out, fold, gf_prepare(to_gf(r)), to_gf(r), use_tab, (gf128*)fo, (gf128*)bo,
      (gf128*)partials);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_lig_intro_eq(const void* f, size_t n, const void* lo, const void* hi, int lo_bits, void* partials,
                              int grid, cudaStream_t st) {
  lig_intro_eq_kernel<<<grid, LG_THREADS, 0, st>>>((const gf128*)f, n, (const gf128*)lo, (const gf128*)hi, lo_bits,
                                                   (gf128*)partials); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_glue_eq(void* b, size_t n, const void* lo, const void* hi, int lo_bits, const uint64_t beta[2],
                         cudaStream_t st) {
  glue_eq_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>((gf128*)b, n, (const gf128*)lo, (const gf128*)hi,
                                                             lo_bits, to_gf(beta)); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_glue(void* b, const void* add, size_t n, const uint64_t beta[2], cudaStream_t st) {
  glue_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>((gf128*)b, (const gf128*)add, n, to_gf(beta)); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

// byte-table path from 2^18 entries: CTAs of 2^10 entries at 2^18, of 2^11
// above (at least 256 CTAs; 2^11 measured faster than 2^10 and 2^9 at 2^19)
constexpr int kBasisTabMinBits = 18;
constexpr int kBasisSlices = 8;
size_t flock_induce_basis_scratch_bytes(int n) { return n >= kBasisTabMinBits ? 0 : ((size_t)kBasisSlices << n) * 16; }

int flock_induce_basis_lo_bits(int n) { return n >= kBasisTabMinBits ? (n == kBasisTabMinBits ? 10 : 11) : (n + 1) / 2; }

int flock_launch_induce_basis(const uint32_t* d_queries, int nq, int n, const void* what_lin, const void* alpha_w,
                              void* W, void* LO, void* HI, void* basis, void* scratch, cudaStream_t st) {
  what_kernel<<<(unsigned)(((size_t)nq * n + 127) / 128), 128, 0, st>>>(d_queries, nq, n, (const gf128*)what_lin,
                                                                          (gf128*)W); flock_count_launch();
  const int lo_bits = flock_induce_basis_lo_bits(n), hi_bits = n - lo_bits;
  const bool tab = n >= kBasisTabMinBits;
  if (lo_bits > TB_LO + TB_HI || hi_bits > TB_LO + TB_HI) return FLOCK_ERR_SHAPE;
  auto tgrid = [&](int bits) { return (unsigned)((size_t)nq * ((((size_t)1 << bits) + TB_THREADS - 1) / TB_THREADS)); };
  tensor_kernel<<<tgrid(lo_bits), TB_THREADS, 0, st>>>((const gf128*)W, nq, n, 0, lo_bits, (const gf128*)alpha_w,
                                                       (gf128*)LO); flock_count_launch();
  tensor_kernel<<<tgrid(hi_bits), TB_THREADS, 0, st>>>((const gf128*)W, nq, n, lo_bits, hi_bits, nullptr,
                                                       (gf128*)HI); flock_count_launch();
  if (tab) {
    flock_once_per_device((const void*)basis_tab_kernel<10>, [] {
      cudaFuncSetAttribute(basis_tab_kernel<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BT_SMEM);
      cudaFuncSetAttribute(basis_tab_kernel<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BT_SMEM);
    });
    const unsigned grid = (unsigned)((size_t)1 << hi_bits);
    if (lo_bits == 10)
      basis_tab_kernel<10><<<grid, BT_THREADS, BT_SMEM, st>>>((const gf128*)LO, (const gf128*)HI, nq, hi_bits,
                                                              (gf128*)basis);
    else
      basis_tab_kernel<11><<<grid, BT_THREADS, BT_SMEM, st>>>((const gf128*)LO, (const gf128*)HI, nq, hi_bits,
                                                              (gf128*)basis);
  } else {
    // slices of the query sum: about 2^18 threads in all, at most kBasisSlices
    // (one thread per entry ran 106 dependent products at 2^16 entries)
    int slices = 1;
    while (slices < kBasisSlices && ((size_t)slices << n) < ((size_t)1 << 18) && slices < nq) slices *= 2;
    const int q_per = (nq + slices - 1) / slices;
    const dim3 grid(grid_for((size_t)1 << n, 256, 152 * 8), slices);
    basis_kernel<<<grid, 256, 0, st>>>((const gf128*)LO, (const gf128*)HI, nq, lo_bits, hi_bits, q_per,
                                       (gf128*)(slices > 1 ? scratch : basis));
    flock_count_launch();
    if (cudaGetLastError() != cudaSuccess) return FLOCK_ERR_CUDA;
    if (slices > 1) return flock_launch_reduce_rows(scratch, slices, 1 << n, basis, st);
    return FLOCK_OK;
  }
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_gather_rows(const void* mat, const uint32_t* rows, int n_rows, int width, void* out,
                             cudaStream_t st) {
  size_t n = (size_t)n_rows * width;
  gather_rows_kernel<<<grid_for(n, 256, 1u << 30), 256, 0, st>>>((const gf128*)mat, rows, n_rows, width,
                                                                  (gf128*)out); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_gather_nodes(const void* tree, const uint32_t* idx, int n, void* out, cudaStream_t st) {
  if (n == 0) return FLOCK_OK;
  gather_nodes_kernel<<<(2 * n + 255) / 256, 256, 0, st>>>((const uint4*)tree, idx, n, (uint4*)out); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_fold_lsb(const void* in, size_t n_out, const uint64_t r[2], void* out, cudaStream_t st) {
  fold_lsb_kernel<<<grid_for(n_out, 256, 152 * 8), 256, 0, st>>>((const gf128*)in, n_out, gf_prepare(to_gf(r)),
                                                                 (gf128*)out);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

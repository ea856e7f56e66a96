// Ring-switch kernels of the PCS opening (crates/flock-core/src/pcs/ring_switch.rs).
//
//  * s_hat_v[b] = sum_pos bit_b(z[pos]) t(pos), t = eq(suffix) (ring_switch.rs:1568-1620):
//    t(pos) = t_lo[pos & lo_mask] * t_hi[pos >> lo_bits]; each warp handles
//    whole hi blocks, folding eight positions at a time through a 256-entry
//    subset-sum table of t_lo, and multiplies its 128 accumulators by t_hi once
//    per block. Lane l owns bits 4l..4l+3.
//  * combined basis b[pos] = sum_k gamma_k sum_b bit_b(t_k(pos)) eq(r''_k)[b]
//    (ring_switch.rs:1720-1760, pcs.rs:1080-1110): 16 byte tables per claim with
//    gamma folded in, one F128 multiply per claim per position.
#include "flock_internal.h"
#include "gf128.cuh"

namespace {

constexpr int SH_THREADS = 256;

__global__ void __launch_bounds__(SH_THREADS)
s_hat_v_kernel(const gf128* __restrict__ z, size_t n, const gf128* __restrict__ t_lo,
               const gf128* __restrict__ t_hi, int lo_bits, gf128* __restrict__ partials) {
  __shared__ gf128 tabs[SH_THREADS / 32][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  gf128* tab = tabs[warp];
  const size_t lo_n = (size_t)1 << lo_bits;
  const size_t n_hi = n >> lo_bits;
  gf128 tot[4];
#pragma unroll
  for (int q = 0; q < 4; q++) tot[q] = gf_zero();
  const size_t gw = (size_t)blockIdx.x * (SH_THREADS / 32) + warp;
  const size_t nw = (size_t)gridDim.x * (SH_THREADS / 32);
  const int word = lane >> 3, shift = (lane & 7) * 4;  // bits 4*lane .. 4*lane+3
  for (size_t h = gw; h < n_hi; h += nw) {
    gf128 acc[4];
#pragma unroll
    for (int q = 0; q < 4; q++) acc[q] = gf_zero();
    for (size_t g = 0; g < lo_n; g += 8) {
      // subset-sum table of t_lo[g..g+8): 8 entries per lane
      __syncwarp();
#pragma unroll
      for (int k = 0; k < 8; k++) {
        int v = lane * 8 + k;
        gf128 s = gf_zero();
#pragma unroll
        for (int r = 0; r < 8; r++)
          if ((v >> r) & 1) s = gf_add(s, t_lo[g + r]);
        tab[v] = s;
      }
      __syncwarp();
      uint32_t nib[8];
#pragma unroll
      for (int r = 0; r < 8; r++) nib[r] = (reinterpret_cast<const uint32_t*>(&z[h * lo_n + g + r])[word] >> shift) & 15;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        uint32_t byte = 0;
#pragma unroll
        for (int r = 0; r < 8; r++) byte |= ((nib[r] >> q) & 1) << r;
        if (byte) acc[q] = gf_add(acc[q], tab[byte]);
      }
    }
    gf128 e = t_hi[h];
#pragma unroll
    for (int q = 0; q < 4; q++) tot[q] = gf_add(tot[q], gf_mul(acc[q], e));
  }
  gf128* out = partials + gw * 128 + 4 * lane;
#pragma unroll
  for (int q = 0; q < 4; q++) out[q] = tot[q];
}

constexpr int CB_THREADS = 256;
// tables: [2][16][256] F128 (gamma-scaled byte tables of eq(r''_k)).
__global__ void __launch_bounds__(CB_THREADS)
combined_basis_kernel(size_t n, const gf128* __restrict__ t0_lo, const gf128* __restrict__ t0_hi,
                      const gf128* __restrict__ t1_lo, const gf128* __restrict__ t1_hi, int lo_bits,
                      const gf128* __restrict__ tables, gf128* __restrict__ b) {
  extern __shared__ gf128 tab[];
  for (int i = threadIdx.x; i < 2 * 16 * 256; i += CB_THREADS) tab[i] = tables[i];
  __syncthreads();
  const size_t lo_mask = ((size_t)1 << lo_bits) - 1;
  for (size_t p = (size_t)blockIdx.x * CB_THREADS + threadIdx.x; p < n; p += (size_t)gridDim.x * CB_THREADS) {
    gf128 u0 = gf_mul(t0_lo[p & lo_mask], t0_hi[p >> lo_bits]);
    gf128 u1 = gf_mul(t1_lo[p & lo_mask], t1_hi[p >> lo_bits]);
    gf128 acc = gf_zero();
#pragma unroll
    for (int q = 0; q < 16; q++) {
      uint32_t b0 = (u0.w[q >> 2] >> (8 * (q & 3))) & 255;
      uint32_t b1 = (u1.w[q >> 2] >> (8 * (q & 3))) & 255;
      acc = gf_add(acc, tab[q * 256 + b0]);
      acc = gf_add(acc, tab[4096 + q * 256 + b1]);
    }
    b[p] = acc;
  }
}

// s_hat_v of the ab claim from lincheck's pre-sumcheck z_vec (ring_switch.rs:1275-1325):
// packed word pos = outer * 128 + (i >> 7), bit b = i & 127, so
// s_hat_v[b] = sum_{h < 128} eq_tail[h] * z_vec[h * 128 + b].
__global__ void shv_from_zvec_kernel(const gf128* __restrict__ zvec, const gf128* __restrict__ eq_tail,
                                     gf128* __restrict__ out) {
  int b = threadIdx.x;
  gf256 acc = {{0, 0, 0, 0}};
  for (int h = 0; h < 128; h++) gf256_acc(acc, gf_mul_wide(eq_tail[h], zvec[h * 128 + b]));
  out[b] = gf256_reduce(acc);
}

}  // namespace

int flock_launch_shv_from_zvec(const void* zvec, const void* eq_tail, void* out, cudaStream_t st) {
  shv_from_zvec_kernel<<<1, 128, 0, st>>>((const gf128*)zvec, (const gf128*)eq_tail, (gf128*)out);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_s_hat_v(const void* z, size_t n, const void* t_lo, const void* t_hi, int lo_bits, void* partials,
                         int grid, cudaStream_t st) {
  s_hat_v_kernel<<<grid, SH_THREADS, 0, st>>>((const gf128*)z, n, (const gf128*)t_lo, (const gf128*)t_hi, lo_bits,
                                              (gf128*)partials); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}
int flock_s_hat_v_warps(int grid) { return grid * (SH_THREADS / 32); }

int flock_launch_combined_basis(size_t n, const void* t0_lo, const void* t0_hi, const void* t1_lo, const void* t1_hi,
                                int lo_bits, const void* tables, void* b, cudaStream_t st) {
  size_t smem = 2 * 16 * 256 * 16;
  flock_once_per_device((const void*)combined_basis_kernel, [] {
    cudaFuncSetAttribute(combined_basis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(2 * 16 * 256 * 16));
  });
  size_t grid = (n + CB_THREADS - 1) / CB_THREADS;
  if (grid > 152 * 2) grid = 152 * 2;
  combined_basis_kernel<<<(unsigned)grid, CB_THREADS, smem, st>>>(
      n, (const gf128*)t0_lo, (const gf128*)t0_hi, (const gf128*)t1_lo, (const gf128*)t1_hi, lo_bits,
      (const gf128*)tables, (gf128*)b); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

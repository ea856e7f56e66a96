// Ring-switch kernels of the PCS opening (crates/flock-core/src/pcs/ring_switch.rs).
//
//  * s_hat_v of the ab claim from lincheck's z_vec (ring_switch.rs:1275-1325);
//    the c claim's comes out of zerocheck round 1, so z is never re-read;
//  * combined basis b[pos] = sum_k gamma_k sum_b bit_b(t_k(pos)) eq(r''_k)[b]
//    (ring_switch.rs:1720-1760, pcs.rs:1080-1110), t_k = eq tensor of the
//    claim's suffix: per high index, byte tables of the linear map
//    lo -> L_k(lo * hi), no F128 multiply per position.
#include "flock_internal.h"
#include "gf128.cuh"

namespace {

constexpr int CB_THREADS = 256;  // at least 256: the table build's first phase takes one thread per image
#ifndef CBM_THREADS
#define CBM_THREADS 512
#endif
constexpr size_t CB_SMEM = (size_t)2 * 16 * 256 * 16 + 2 * 128 * 16;

// x^i * h for 0 <= i < 128: shift into 256 bits, then reduce.
__device__ __forceinline__ gf128 gf_mul_xpow(gf128 h, int i) {
  uint64_t lo = h.w[0] | ((uint64_t)h.w[1] << 32), hi = h.w[2] | ((uint64_t)h.w[3] << 32);
  uint64_t r[4] = {0, 0, 0, 0};
  // (hi:lo) << i over four 64-bit words
  const int wsh = i >> 6, bsh = i & 63;
  uint64_t s0 = lo << bsh, s1 = (hi << bsh) | (bsh ? lo >> (64 - bsh) : 0), s2 = bsh ? hi >> (64 - bsh) : 0;
  if (wsh == 0) { r[0] = s0; r[1] = s1; r[2] = s2; }
  else { r[1] = s0; r[2] = s1; r[3] = s2; }
  return gf_reduce(r[0], r[1], r[2], r[3]);
}

// Combined basis b[p] = sum_k L_k(lo_k[p & lo_mask] * hi_k[p >> lo_bits]) with
// the GF(2)-linear map L_k(u) = sum_b bit_b(u) w_k[b], w_k = gamma_k eq(r''_k)
// (ring_switch.rs:1720-1760, pcs.rs:1080-1110). For a fixed high index the
// map lo -> L_k(lo * h) is again GF(2)-linear, so a CTA builds its sixteen
// byte tables from the 128 images L_k(x^i h) and then needs no GF(2^128)
// product per position: 2 x 16 table lookups. Each CTA owns one high index
// and a slice of the low range.
// The sixteen byte tables of both claims for high index h (tab: [2][256 v][16 q],
// entry (k, v, q) in bank group q mod 8; beta: [2][8 t][16 q] scratch).
__device__ __forceinline__ void cb_build_tables(size_t h, const gf128* __restrict__ hi0, const gf128* __restrict__ hi1,
                                                const gf128* __restrict__ w, gf128* tab, gf128* beta) {
  if (threadIdx.x < 256) {
    const int k = threadIdx.x >> 7, i = threadIdx.x & 127;
    const gf128 y = gf_mul_xpow(k ? hi1[h] : hi0[h], i);
    const gf128* wk = w + 128 * k;
    gf128 acc = gf_zero();
#pragma unroll 4
    for (int bb = 0; bb < 128; bb++)
      if ((y.w[bb >> 5] >> (bb & 31)) & 1) acc = gf_add(acc, wk[bb]);
    beta[k * 128 + (i & 7) * 16 + (i >> 3)] = acc;
  }
  __syncthreads();
  // subset sums by a Gray walk: item (k, c, q) owns entries v = 8c .. 8c+7 of
  // position q of claim k, starts from the sum over the bits of 8c and adds
  // one image per entry (consecutive items: consecutive q, distinct banks)
  for (int it = threadIdx.x; it < 2 * 32 * 16; it += blockDim.x) {
    const int q = it & 15, c = (it >> 4) & 31, k = it >> 9;
    const gf128* bq = beta + k * 128 + q;
    gf128 acc = gf_zero();
#pragma unroll
    for (int t = 3; t < 8; t++)
      if ((c >> (t - 3)) & 1) acc = gf_add(acc, bq[16 * t]);
    gf128* row = tab + k * 4096 + q;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      if (i) acc = gf_add(acc, bq[16 * ((i & 1) ? 0 : (i & 2) ? 1 : 2)]);
      row[(8 * c + (i ^ (i >> 1))) << 4] = acc;
    }
  }
  __syncthreads();
}

// The bytes of u permuted so that byte st of p is byte st ^ rot of u (rot < 16):
// a half swap for bit 3 of rot, a word swap for bit 2, a byte permutation
// within each word for bits 0..1.
__device__ __forceinline__ void cb_permute(const gf128& u, int rot, uint32_t p[4]) {
  const bool s8 = rot & 8, s4 = rot & 4;
  const uint32_t a0 = s8 ? u.w[2] : u.w[0], a1 = s8 ? u.w[3] : u.w[1];
  const uint32_t a2 = s8 ? u.w[0] : u.w[2], a3 = s8 ? u.w[1] : u.w[3];
  const uint32_t x3 = rot & 3;
  const uint32_t sel = x3 == 0 ? 0x3210u : x3 == 1 ? 0x2301u : x3 == 2 ? 0x1032u : 0x0123u;
  p[0] = __byte_perm(s4 ? a1 : a0, 0, sel);
  p[1] = __byte_perm(s4 ? a0 : a1, 0, sel);
  p[2] = __byte_perm(s4 ? a3 : a2, 0, sel);
  p[3] = __byte_perm(s4 ? a2 : a3, 0, sel);
}

// b[p] for the low indices u0 = lo0[j], u1 = lo1[j]: 2 x 16 table lookups.
// At step st a lane reads byte position q = st ^ rot (rot = lane mod 16), so
// eight consecutive lanes read eight distinct bank groups (entry (v, q) is
// 16-byte slot 16 v + q: bank group q mod 8) and the random lookups are
// conflict-free. The bytes are permuted once to that order (cb_permute), so
// each step is a byte move, one logic op for the slot offset, the load and the
// XORs, with no position-dependent word select or shift.
__device__ __forceinline__ gf128 cb_value(const gf128* tab, const gf128 u0, const gf128 u1, int rot) {
  uint32_t p0[4], p1[4];
  cb_permute(u0, rot, p0);
  cb_permute(u1, rot, p1);
  const char* base = reinterpret_cast<const char*>(tab);
  const uint32_t xk = (uint32_t)rot << 4;  // byte offset of the position XOR
  uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll
  for (int st = 0; st < 16; st++) {
    // byte st of p at bits 8..15 = v << 8: slot (v << 4) | (st ^ rot) is byte
    // offset (v << 8) | ((st ^ rot) << 4); claim 1's table is 4096 slots on
    const uint32_t sh = 0x4404u | ((uint32_t)(st & 3) << 4);
    const uint32_t o0 = (__byte_perm(p0[st >> 2], 0, sh) | ((uint32_t)st << 4)) ^ xk;
    const uint32_t o1 = (__byte_perm(p1[st >> 2], 0, sh) | ((uint32_t)st << 4)) ^ xk;
    const uint4 t0 = *reinterpret_cast<const uint4*>(base + o0);
    const uint4 t1 = *reinterpret_cast<const uint4*>(base + 4096 * 16 + o1);
    a0 ^= t0.x ^ t1.x;
    a1 ^= t0.y ^ t1.y;
    a2 ^= t0.z ^ t1.z;
    a3 ^= t0.w ^ t1.w;
  }
  gf128 r;
  r.w[0] = a0; r.w[1] = a1; r.w[2] = a2; r.w[3] = a3;
  return r;
}

__global__ void __launch_bounds__(CB_THREADS)
combined_basis_kernel(int lo_bits, int slices, const gf128* __restrict__ lo0, const gf128* __restrict__ hi0,
                      const gf128* __restrict__ lo1, const gf128* __restrict__ hi1, const gf128* __restrict__ w,
                      gf128* __restrict__ b) {
  extern __shared__ gf128 cb[];
  gf128* tab = cb;
  gf128* beta = cb + 2 * 16 * 256;
  const size_t h = blockIdx.x / slices;
  const int slice = blockIdx.x % slices;
  cb_build_tables(h, hi0, hi1, w, tab, beta);
  const size_t lo_n = (size_t)1 << lo_bits;
  const size_t per = lo_n / slices;
  const size_t j0 = (size_t)slice * per;
  const int rot = threadIdx.x & 15;
  for (size_t j = j0 + threadIdx.x; j < j0 + per; j += CB_THREADS) b[(h << lo_bits) + j] = cb_value(tab, lo0[j], lo1[j], rot);
}

// The combined basis fused with the first message of the Ligerito sumcheck
// over (f, b) (ligerito.rs:6222-6300, as lig_fold_msg without a fold):
// u0 = sum f[2q] b[2q], u2 = sum (f[2q] + f[2q+1]) (b[2q] + b[2q+1]). A thread
// takes position pairs: the basis values come from the table lookups (load
// and store pipes) and the two products from the carry-less multiply (integer
// pipes) of the same pass, so the two overlap and b is not read back.
// Partials: (u0, u2, 0) per block.
__global__ void __launch_bounds__(CBM_THREADS)
combined_basis_msg_kernel(int lo_bits, int slices, const gf128* __restrict__ lo0, const gf128* __restrict__ hi0,
                          const gf128* __restrict__ lo1, const gf128* __restrict__ hi1, const gf128* __restrict__ w,
                          const gf128* __restrict__ f, gf128* __restrict__ b, gf128* __restrict__ partials) {
  extern __shared__ gf128 cb[];
  gf128* tab = cb;
  gf128* beta = cb + 2 * 16 * 256;
  const size_t h = blockIdx.x / slices;
  const int slice = blockIdx.x % slices;
  cb_build_tables(h, hi0, hi1, w, tab, beta);
  const size_t lo_n = (size_t)1 << lo_bits;
  const size_t per = lo_n / slices;
  const size_t j0 = (size_t)slice * per;
  const int rot = threadIdx.x & 15;
  gf256 u0 = {{0, 0, 0, 0}}, u2 = u0;
  for (size_t j = j0 + 2 * threadIdx.x; j < j0 + per; j += 2 * CBM_THREADS) {
    const size_t p = (h << lo_bits) + j;
    const gf128 b0 = cb_value(tab, lo0[j], lo1[j], rot), b1 = cb_value(tab, lo0[j + 1], lo1[j + 1], rot ^ 8);
    b[p] = b0;
    b[p + 1] = b1;
    const gf128 f0 = f[p], f1 = f[p + 1];
    gf256_acc(u0, gf_mul_wide(f0, b0));
    gf256_acc(u2, gf_mul_wide(gf_add(f0, f1), gf_add(b0, b1)));
  }
  __shared__ gf256 red[2][CBM_THREADS / 32];
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      u0.r[k] ^= __shfl_xor_sync(0xffffffffu, u0.r[k], off);
      u2.r[k] ^= __shfl_xor_sync(0xffffffffu, u2.r[k], off);
    }
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][wid] = u0;
    red[1][wid] = u2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    gf256 s0 = {{0, 0, 0, 0}}, s1 = s0;
    for (int k = 0; k < CBM_THREADS / 32; k++) {
      gf256_acc(s0, red[0][k]);
      gf256_acc(s1, red[1][k]);
    }
    partials[3 * blockIdx.x] = gf256_reduce(s0);
    partials[3 * blockIdx.x + 1] = gf256_reduce(s1);
    partials[3 * blockIdx.x + 2] = gf_zero();
  }
}

// s_hat_v of the ab claim from lincheck's pre-sumcheck z_vec (ring_switch.rs:1275-1325):
// packed word pos = outer * 128 + (i >> 7), bit b = i & 127, so
// s_hat_v[b] = sum_{h < 128} eq_tail[h] * z_vec[h * 128 + b].
// SHV_CTAS CTAs of 512 threads, CTA g taking h in [4 g, 4 g + 4): thread
// (q, b) forms one product, the four of each b are XORed in shared memory
// into row g of the partials, which a row reduction then folds (one CTA
// forming all 16 K products took 58 us, latency-bound on one SM).
constexpr int SHV_CTAS = 32;
__global__ void __launch_bounds__(512)
shv_from_zvec_kernel(const gf128* __restrict__ zvec, const gf128* __restrict__ eq_tail, gf128* __restrict__ part) {
  __shared__ gf128 red[4][128];
  const int b = threadIdx.x & 127, q = threadIdx.x >> 7;
  const int h = 4 * blockIdx.x + q;
  red[q][b] = gf_mul(eq_tail[h], zvec[h * 128 + b]);
  __syncthreads();
  if (q == 0) {
    gf128 v = red[0][b];
    for (int k = 1; k < 4; k++) v = gf_add(v, red[k][b]);
    part[(size_t)blockIdx.x * 128 + b] = v;
  }
}

}  // namespace

int flock_launch_shv_from_zvec(const void* zvec, const void* eq_tail, void* scratch, void* out, cudaStream_t st) {
  static_assert(SHV_CTAS * 4 == 128, "the CTAs cover the 128 high indices");
  shv_from_zvec_kernel<<<SHV_CTAS, 512, 0, st>>>((const gf128*)zvec, (const gf128*)eq_tail, (gf128*)scratch);
  flock_count_launch();
  if (cudaGetLastError() != cudaSuccess) return FLOCK_ERR_CUDA;
  return flock_launch_reduce_rows(scratch, SHV_CTAS, 128, out, st);
}


namespace {
// CTAs per high index: enough CTAs to fill the GPU, splitting the low range
// when there are few high indices.
int cb_slices(size_t n_hi, size_t lo_n) {
  int slices = 1;
  while (n_hi * slices < 152 * 2 && lo_n / (2 * slices) >= CB_THREADS) slices *= 2;
  return slices;
}
}  // namespace

int flock_launch_combined_basis(size_t n, const void* t0_lo, const void* t0_hi, const void* t1_lo, const void* t1_hi,
                                int lo_bits, const void* w, void* b, cudaStream_t st) {
  flock_once_per_device((const void*)combined_basis_kernel, [] {
    cudaFuncSetAttribute(combined_basis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CB_SMEM);
  });
  const size_t lo_n = (size_t)1 << lo_bits;
  if (n % lo_n != 0 || lo_n < CB_THREADS) return FLOCK_ERR_SHAPE;
  const size_t n_hi = n >> lo_bits;
  const int slices = cb_slices(n_hi, lo_n);
  combined_basis_kernel<<<(unsigned)(n_hi * slices), CB_THREADS, CB_SMEM, st>>>(
      lo_bits, slices, (const gf128*)t0_lo, (const gf128*)t0_hi, (const gf128*)t1_lo, (const gf128*)t1_hi,
      (const gf128*)w, (gf128*)b);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_combined_basis_msg_grid(size_t n, int lo_bits) {
  const size_t lo_n = (size_t)1 << lo_bits, n_hi = n >> lo_bits;
  return (int)(n_hi * cb_slices(n_hi, lo_n));
}

int flock_launch_combined_basis_msg(size_t n, const void* t0_lo, const void* t0_hi, const void* t1_lo,
                                    const void* t1_hi, int lo_bits, const void* w, const void* f, void* b,
                                    void* partials, cudaStream_t st) {
  flock_once_per_device((const void*)combined_basis_msg_kernel, [] {
    cudaFuncSetAttribute(combined_basis_msg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CB_SMEM);
  });
  const size_t lo_n = (size_t)1 << lo_bits;
  if (n % lo_n != 0 || lo_n < CB_THREADS) return FLOCK_ERR_SHAPE;
  const size_t n_hi = n >> lo_bits;
  const int slices = cb_slices(n_hi, lo_n);
  if ((lo_n / slices) % 2) return FLOCK_ERR_SHAPE;
  combined_basis_msg_kernel<<<(unsigned)(n_hi * slices), CBM_THREADS, CB_SMEM, st>>>(
      lo_bits, slices, (const gf128*)t0_lo, (const gf128*)t0_hi, (const gf128*)t1_lo, (const gf128*)t1_hi,
      (const gf128*)w, (const gf128*)f, (gf128*)b, (gf128*)partials);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

// Zerocheck kernels: univariate-skip round 1 and the multilinear rounds.
//
// Protocol: crates/flock-core/src/zerocheck.rs:482-1360 (verifier :1365-1517).
// Round 1 sends, for the 64 points lambda_i = 64 + i of GF(2^8) (embedded by
// phi8), P^AB(l) = sum_x eq(r_rest, x) phi8(a^(l,x) b^(l,x)) and
// P^C(l) = sum_x eq(r_rest, x) phi8(c^(l,x)), where a^(., x) is the degree<64
// extension of the 64 witness bits of row x from S = {0..63}
// (zerocheck/univariate_skip.rs:84-138).
//
// GB300 formulation. The first seven rest variables carry fixed challenges
// (zerocheck/univariate_skip_optimized.rs:85-130): three phi8 constants and
// four g/(1+g) with g = x^(2^j). Their eq weight factors as
//   eq_in(xs, xm) = phi8(e8[xs]) * x^xm * Dinv,
// so per outer index xo (128 rows) the kernel needs no F128 multiply until
//   V_i(xo) = sum_xm x^xm phi8( sum_xs e8[xs] * y_i(xs, xm, xo) ),
// which is a 143-bit shifted XOR of table values, reduced once and multiplied
// by eq_out(xo). The F8 values y_i = a^_i b^_i are computed bit-sliced over the
// 64 lambda points (eight 64-bit planes), so one product handles all points.
// P^C uses linearity: it needs only the 128 sums
//   S[64t + s] = sum_{x : x&1 = t} eq(r[7..m], x >> 1) c_s(x)
// (C_s = (1 + r6) S[s] + r6 S[64 + s], mapped to Lambda on the host), and S is
// exactly the ring-switch statistic s_hat_v of the c-claim (bit 64t + s of
// packed word x >> 1), so the opening reuses it.
#include <algorithm>

#include "flock_internal.h"
#include "gf128.cuh"
#include "gf_tab.cuh"
#include "zc_tables.h"

namespace {

#ifndef ZC1_THREADS
#define ZC1_THREADS 384
#endif
constexpr int R1_THREADS = ZC1_THREADS;  // 12 warps, one block per SM
#ifndef ZC1_PAR_UNROLL
#define ZC1_PAR_UNROLL 1
#endif
constexpr int kZc1ParUnroll = ZC1_PAR_UNROLL;  // 1: one loop body for both row parities

// 143-bit accumulator (five 32-bit words) for shifted table values.
struct Acc5 {
  uint32_t w[5];
};

__device__ __forceinline__ gf128 acc_reduce(const Acc5& a) {
  // bits 128..143 live in w[4] (< 2^15): fold with x^128 = x^7 + x^2 + x + 1
  uint32_t ov = a.w[4];
  uint32_t f = ov ^ (ov << 1) ^ (ov << 2) ^ (ov << 7);  // < 2^22, no further overflow
  gf128 r;
  r.w[0] = a.w[0] ^ f;
  r.w[1] = a.w[1];
  r.w[2] = a.w[2];
  r.w[3] = a.w[3];
  return r;
}

// Bit-sliced GF(2^8) product of 64 lane pairs (planes p[j] = bit j over lanes).
__device__ __forceinline__ void f8_mul_planes(const uint64_t* a, const uint64_t* b, uint64_t* out) {
  uint64_t p[15];
#pragma unroll
  for (int k = 0; k < 15; k++) p[k] = 0;
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) p[i + j] ^= a[i] & b[j];
#pragma unroll
  for (int k = 14; k >= 8; k--) {
    p[k - 4] ^= p[k];
    p[k - 5] ^= p[k];
    p[k - 7] ^= p[k];
    p[k - 8] ^= p[k];
  }
#pragma unroll
  for (int k = 0; k < 8; k++) out[k] = p[k];
}

// GF(2^8) product (modulus x^8 + x^4 + x^3 + x + 1), usable in constant
// expressions so that multiplications by the fixed challenges below fold into
// compile-time XOR patterns.
__host__ __device__ constexpr uint8_t f8_mul_c(uint8_t a, uint8_t b) {
  unsigned acc = 0;
  for (int i = 0; i < 8; i++)
    if ((a >> i) & 1) acc ^= (unsigned)b << i;
  for (int i = 14; i >= 8; i--)
    if ((acc >> i) & 1) acc ^= 0x11Bu << (i - 8);
  return (uint8_t)acc;
}

// eq factor of one fixed small challenge: bit ? C : 1 + C.
__host__ __device__ constexpr uint8_t f8_eq_factor(int v, int bit) {
  return bit ? zc::SMALL_CHAL[v] : (uint8_t)(1 ^ zc::SMALL_CHAL[v]);
}

// acc (+)= E * y on bit-sliced planes, E a compile-time GF(2^8) constant: plane
// j takes y_k where bit j of E x^k is set (about half of the 64 pairs).
template <uint8_t E, bool ADD>
__device__ __forceinline__ void f8_mul_const_planes(const uint64_t y[8], uint64_t acc[8]) {
#pragma unroll
  for (int j = 0; j < 8; j++) {
    uint64_t s = ADD ? acc[j] : 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if ((f8_mul_c(E, (uint8_t)(1u << k)) >> j) & 1) s ^= y[k];
    acc[j] = s;
  }
}

// 8x8 bit-matrix transpose: bit 8r + c <-> bit 8c + r.
__device__ __forceinline__ uint64_t transpose8x8(uint64_t x) {
  uint64_t t;
  t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull; x = x ^ t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull; x = x ^ t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull; x = x ^ t ^ (t << 28);
  return x;
}

// Eight 64-bit planes -> bytes 32 h .. 32 h + 31 of the 64 (byte i = sum_j
// bit i of p[j] << j), as words 8 h .. 8 h + 7 of dst (word k holds bytes
// 4k .. 4k+3), written with two 16-byte stores: the two half-warps holding
// the same planes produce one half of the bytes each.
__device__ __forceinline__ void planes_to_bytes_half(const uint64_t p[8], uint32_t* dst, int h) {
  uint32_t q[8];
#pragma unroll
  for (int j = 0; j < 8; j++) q[j] = h ? (uint32_t)(p[j] >> 32) : (uint32_t)p[j];
  uint32_t o[8];
#pragma unroll
  for (int b = 0; b < 4; b++) {
    // byte j of x = byte b of q[j]
    const uint32_t sel = (uint32_t)b | ((uint32_t)(b + 4) << 4);
    const uint32_t lo = __byte_perm(__byte_perm(q[0], q[1], sel), __byte_perm(q[2], q[3], sel), 0x5410);
    const uint32_t hi = __byte_perm(__byte_perm(q[4], q[5], sel), __byte_perm(q[6], q[7], sel), 0x5410);
    const uint64_t y = transpose8x8(((uint64_t)hi << 32) | lo);
    o[2 * b] = (uint32_t)y;
    o[2 * b + 1] = (uint32_t)(y >> 32);
  }
  uint4* d = reinterpret_cast<uint4*>(dst + 8 * h);
  d[0] = make_uint4(o[0], o[1], o[2], o[3]);
  d[1] = make_uint4(o[4], o[5], o[6], o[7]);
}

// a ^= v << sh for 0 <= sh < 16, branch-free.
__device__ __forceinline__ void acc_shift_xor_v(Acc5& a, const uint4 v, uint32_t sh) {
  a.w[0] ^= v.x << sh;
  a.w[1] ^= __funnelshift_l(v.x, v.y, sh);
  a.w[2] ^= __funnelshift_l(v.y, v.z, sh);
  a.w[3] ^= __funnelshift_l(v.z, v.w, sh);
  a.w[4] ^= __funnelshift_l(v.w, 0u, sh);
}

// 288-bit accumulator of shifted unreduced products (a 256-bit carry-less
// product shifted by < 16 bits): the reduction is paid once per sum.
struct Acc9 {
  uint32_t w[9];
};

__device__ __forceinline__ void acc9_shift_xor(Acc9& a, const gf256& v, uint32_t sh) {
  uint32_t u[8];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    u[2 * k] = (uint32_t)v.r[k];
    u[2 * k + 1] = (uint32_t)(v.r[k] >> 32);
  }
  a.w[0] ^= u[0] << sh;
#pragma unroll
  for (int k = 1; k < 8; k++) a.w[k] ^= __funnelshift_l(u[k - 1], u[k], sh);
  a.w[8] ^= __funnelshift_l(u[7], 0u, sh);
}

// a mod x^128 + x^7 + x^2 + x + 1 for a below 2^272: the high part H (bits
// 128 and up, below 2^144) folds in as H (1 + x + x^2 + x^7), whose bits
// above 127 (fewer than 23) fold in once more.
__device__ __forceinline__ gf128 acc9_reduce(const Acc9& a) {
  const uint64_t l0 = a.w[0] | ((uint64_t)a.w[1] << 32), l1 = a.w[2] | ((uint64_t)a.w[3] << 32);
  const uint64_t h0 = a.w[4] | ((uint64_t)a.w[5] << 32), h1 = a.w[6] | ((uint64_t)a.w[7] << 32), h2 = a.w[8];
  const uint64_t t0 = h0 ^ (h0 << 1) ^ (h0 << 2) ^ (h0 << 7);
  const uint64_t t1 = h1 ^ ((h1 << 1) | (h0 >> 63)) ^ ((h1 << 2) | (h0 >> 62)) ^ ((h1 << 7) | (h0 >> 57));
  const uint64_t t2 = h2 ^ ((h2 << 1) | (h1 >> 63)) ^ ((h2 << 2) | (h1 >> 62)) ^ ((h2 << 7) | (h1 >> 57));
  const uint64_t lo = l0 ^ t0 ^ t2 ^ (t2 << 1) ^ (t2 << 2) ^ (t2 << 7), hi = l1 ^ t1;
  gf128 r;
  r.w[0] = (uint32_t)lo; r.w[1] = (uint32_t)(lo >> 32); r.w[2] = (uint32_t)hi; r.w[3] = (uint32_t)(hi >> 32);
  return r;
}

// One 16-byte shared-memory load as a single 128-bit access. The extension
// lookups below are conflict-free only as 128-bit accesses (quarter-warp
// phases over eight distinct bank groups); split into two 64-bit loads, a
// half-warp phase would pair lanes l and l + 8 on the same banks.
__device__ __forceinline__ uint4 lds128(const uint4* p) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"((uint32_t)__cvta_generic_to_shared(p)));
  return v;
}

__device__ __forceinline__ uint64_t shfl_xor64(uint64_t v, int m) {
  const uint32_t lo = __shfl_xor_sync(0xffffffffu, (uint32_t)v, m);
  const uint32_t hi = __shfl_xor_sync(0xffffffffu, (uint32_t)(v >> 32), m);
  return ((uint64_t)hi << 32) | lo;
}

// Shared memory of the round-1 kernel (32-bit words):
//   ext  [4 quarters q][256 values v][8 byte positions c] of 16 B (a value's
//        eight 64-bit planes, quarter q = planes 2q, 2q+1): the table of byte
//        position c lies in bank group c (16-byte slot index = c mod 8), and at
//        step k lane l looks up byte position (l + k) mod 8, so any eight
//        consecutive lanes hit eight distinct bank groups and the random
//        lookups are conflict-free;
//   T8   per warp (one outer block xo per warp at a time): the eq-weighted
//        phi8 table T8[v] = phi8(v) e for the 256 bytes v, e = eq_out(xo)
//        (entry v at slot v), so the block's values come out already
//        weighted and need no GF(2^128) product; the table is the subset
//        sums of its basis phi8(2^k) e, k < 8 (phi8 is additive), which
//        zc1_eq_basis_kernel computes for every block beforehand. One lookup per
//        value: the random bytes of a quarter warp share bank groups at times
//        (about two wavefronts per quarter-warp lookup, measured), which the
//        load/store pipe absorbs; with two nibble tables L[v & 15] + H[v >> 4] in eight
//        conflict-free replicas (the same 4 KiB) each value took two lookups,
//        two index computations and a four-word XOR on the busy ALU pipe;
//   xch  per warp: [16 producer rows] of 20 words (64 bytes used; the odd
//        80-byte row pitch makes the 16-byte stores conflict-free), one plane
//        set at a time.
// The two half-warps share the outer block: each sums half of its rows, the
// halves add their planes with one exchange of registers, each converts half
// of the points to bytes, and each lane then handles two of the 64 points.
constexpr int R1_ROW = 20;
constexpr int R1_XCH = 16 * R1_ROW;
constexpr int R1_WARPS = R1_THREADS / 32;
constexpr size_t R1_SMEM = (size_t)8 * 4 * 256 * 16 + (size_t)R1_WARPS * 256 * 16 + (size_t)R1_WARPS * R1_XCH * 4;
static_assert(R1_SMEM <= 232448, "round-1 shared memory above the 227 KB per-block limit");

// grid: each warp walks outer blocks; lane: xm = lane & 15 (producer row
// group, then point quad), h = lane >> 4 (row half, then point pair).
__global__ void __launch_bounds__(R1_THREADS, 1)
zc_round1_kernel(const uint64_t* __restrict__ A, const uint64_t* __restrict__ B, const uint64_t* __restrict__ C,
                 size_t n_outer, const uint4* __restrict__ eq_basis, const ZcRound1Tables* __restrict__ T,
                 gf128* __restrict__ partials) {
  extern __shared__ uint4 sm[];
  uint4* ext = sm;                                                   // [4][256][8]
  uint4* t8 = ext + 8 * 4 * 256;                                     // per warp T8[256]
  uint32_t* xch = reinterpret_cast<uint32_t*>(t8 + R1_WARPS * 256);  // per warp [R1_XCH]
  const uint64_t* ext_src = &T->ext[0][0][0];
  for (int i = threadIdx.x; i < 8 * 4 * 256; i += R1_THREADS) {
    const int q = i >> 11, v = (i >> 3) & 255, c = i & 7;
    const uint64_t* e = ext_src + ((size_t)(c * 256 + v) << 3) + 2 * q;
    ext[i] = make_uint4((uint32_t)e[0], (uint32_t)(e[0] >> 32), (uint32_t)e[1], (uint32_t)(e[1] >> 32));
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int xm = lane & 15, h = lane >> 4;
  uint32_t* my_x = xch + warp * R1_XCH;
  uint4* my_t8 = t8 + warp * 256;
  // points 4 xm + 2 h + {0, 1}: a b sums, then c sums of parity 0 and 1
  gf128 sum_ab[2], sum_c[4];
#pragma unroll
  for (int q = 0; q < 2; q++) sum_ab[q] = gf_zero();
#pragma unroll
  for (int q = 0; q < 4; q++) sum_c[q] = gf_zero();

  const size_t total_warps = (size_t)gridDim.x * R1_WARPS;
  for (size_t xo = (size_t)blockIdx.x * R1_WARPS + warp; xo < n_outer; xo += total_warps) {
    uint64_t w[8], t[16];
#pragma unroll
    for (int j = 0; j < 8; j++) w[j] = 0;
#pragma unroll
    for (int j = 0; j < 16; j++) t[j] = 0;
    const size_t row0 = xo * 128 + (size_t)xm * 8 + 4 * h;
#pragma unroll 1
    for (int xs2 = 0; xs2 < 2; xs2++)
#pragma unroll kZc1ParUnroll
      for (int par = 0; par < 2; par++) {
        const int xs = 4 * h + 2 * xs2 + par;
        const uint64_t ra = A[row0 + 2 * xs2 + par], rb = B[row0 + 2 * xs2 + par], rc = C[row0 + 2 * xs2 + par];
        uint64_t ea[8], eb[8];
#pragma unroll
        for (int j = 0; j < 8; j++) { ea[j] = 0; eb[j] = 0; }
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int c = (lane + k) & 7;  // rotated byte position: conflict-free bank groups
          const uint4* pa = ext + ((((uint32_t)(ra >> (8 * c))) & 255) << 3) + c;
          const uint4* pb = ext + ((((uint32_t)(rb >> (8 * c))) & 255) << 3) + c;
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const uint4 va = lds128(pa + q * 2048), vb = lds128(pb + q * 2048);
            ea[2 * q] ^= ((uint64_t)va.y << 32) | va.x;
            ea[2 * q + 1] ^= ((uint64_t)va.w << 32) | va.z;
            eb[2 * q] ^= ((uint64_t)vb.y << 32) | vb.x;
            eb[2 * q + 1] ^= ((uint64_t)vb.w << 32) | vb.z;
          }
        }
        uint64_t y[8];
        f8_mul_planes(ea, eb, y);
        // w += e8[xs] * y with e8[xs] = f0(par) f1(xs2) f2(h): the row factor
        // f0 f1 is one of four compile-time constants (xs2 and par are the
        // same in every lane, so the switch does not diverge); f2(h) is
        // applied once per block below. t[xs & 1] += e8c[xs >> 1] * c_s
        // (c_s in {0,1}: plane j takes c where bit j of the constant is set).
        switch (2 * xs2 + par) {
          case 0: f8_mul_const_planes<f8_mul_c(f8_eq_factor(0, 0), f8_eq_factor(1, 0)), true>(y, w); break;
          case 1: f8_mul_const_planes<f8_mul_c(f8_eq_factor(0, 1), f8_eq_factor(1, 0)), true>(y, w); break;
          case 2: f8_mul_const_planes<f8_mul_c(f8_eq_factor(0, 0), f8_eq_factor(1, 1)), true>(y, w); break;
          default: f8_mul_const_planes<f8_mul_c(f8_eq_factor(0, 1), f8_eq_factor(1, 1)), true>(y, w); break;
        }
        const uint8_t e8c = T->e8c[xs >> 1];
        // c goes to the parity-par half of t; with the parity a runtime value
        // (one loop body for both parities) the halves take rc or 0
        const uint64_t c_even = par ? 0 : rc, c_odd = par ? rc : 0;
#pragma unroll
        for (int j = 0; j < 8; j++)
          if ((e8c >> j) & 1) {
            t[j] ^= c_even;
            t[8 + j] ^= c_odd;
          }
      }
    // the rows' common factor f2(h) (h differs between the half-warps: both
    // compile-time products, then a select)
    {
      uint64_t w0[8], w1[8];
      f8_mul_const_planes<f8_eq_factor(2, 0), false>(w, w0);
      f8_mul_const_planes<f8_eq_factor(2, 1), false>(w, w1);
#pragma unroll
      for (int j = 0; j < 8; j++) w[j] = h ? w1[j] : w0[j];
    }
    // the two halves' row sums of producer group xm: add them
#pragma unroll
    for (int j = 0; j < 8; j++) w[j] ^= shfl_xor64(w[j], 16);
#pragma unroll
    for (int j = 0; j < 16; j++) t[j] ^= shfl_xor64(t[j], 16);
    // eq-weighted phi8 table of this block (see the layout above)
    {
      // lane l writes T8[l + 32 i], i < 8: the part of bits 0..4 (l) once,
      // then the part of bits 5..7 (i) along a Gray walk, one XOR per entry;
      // a quarter warp's stores are 128 consecutive bytes
      uint4 pb[8];
#pragma unroll
      for (int k = 0; k < 8; k++) pb[k] = eq_basis[xo * 8 + k];
      uint4 lo = make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int k = 0; k < 5; k++) {
        const uint32_t m = 0u - ((uint32_t)(lane >> k) & 1u);
        lo.x ^= pb[k].x & m; lo.y ^= pb[k].y & m; lo.z ^= pb[k].z & m; lo.w ^= pb[k].w & m;
      }
      uint4 hp = make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int g = 0; g < 8; g++) {
        if (g) {
          const uint4 a = pb[5 + ((g & 1) ? 0 : (g & 2) ? 1 : 2)];
          hp.x ^= a.x; hp.y ^= a.y; hp.z ^= a.z; hp.w ^= a.w;
        }
        const int i = g ^ (g >> 1);
        my_t8[lane + 32 * i] = make_uint4(lo.x ^ hp.x, lo.y ^ hp.y, lo.z ^ hp.z, lo.w ^ hp.w);
      }
    }
    // Hand the three plane sets, one at a time, to the lanes as bytes: the
    // lanes of point quad xm read word xm of every producer row, half h
    // taking points 4 xm + 2 h, 4 xm + 2 h + 1.
#pragma unroll 1
    for (int set = 0; set < 3; set++) {
      uint64_t pl[8];
#pragma unroll
      for (int j = 0; j < 8; j++) pl[j] = set == 0 ? w[j] : set == 1 ? t[j] : t[8 + j];
      __syncwarp();
      planes_to_bytes_half(pl, my_x + xm * R1_ROW, h);
      __syncwarp();
      Acc5 v[2];
#pragma unroll
      for (int q = 0; q < 2; q++)
#pragma unroll
        for (int k = 0; k < 5; k++) v[q].w[k] = 0;
#pragma unroll 4
      for (int mm2 = 0; mm2 < 16; mm2++) {
        const uint32_t bw = my_x[mm2 * R1_ROW + xm] >> (16 * h);
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const uint32_t v8 = (bw >> (8 * q)) & 255;
          acc_shift_xor_v(v[q], my_t8[v8], (uint32_t)mm2);
        }
      }
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const gf128 p = acc_reduce(v[q]);
        if (set == 0) sum_ab[q] = gf_add(sum_ab[q], p);
        else if (set == 1) sum_c[q] = gf_add(sum_c[q], p);
        else sum_c[2 + q] = gf_add(sum_c[2 + q], p);
      }
    }
    __syncwarp();
  }
  // reduce the warps of the block in shared memory (reusing the extension
  // tables) and write one row of 192 partial sums per block: 64 P^AB values,
  // then S[0..128).
  __syncthreads();
  gf128* red = reinterpret_cast<gf128*>(ext);  // [warps][192], in the no longer needed extension tables
  {
    gf128* o = red + warp * 192 + 4 * xm + 2 * h;
#pragma unroll
    for (int q = 0; q < 2; q++) {
      o[q] = sum_ab[q];
      o[64 + q] = sum_c[q];
      o[128 + q] = sum_c[2 + q];
    }
  }
  __syncthreads();
  for (int col = threadIdx.x; col < 192; col += R1_THREADS) {
    gf128 acc = gf_zero();
    for (int w2 = 0; w2 < R1_WARPS; w2++) acc = gf_add(acc, red[w2 * 192 + col]);
    partials[(size_t)blockIdx.x * 192 + col] = acc;
  }
}

// The basis of round 1's per-block tables: out[8 xo + k] = phi8(2^k) eq[xo]
// for every outer block xo (eight products per block, all in parallel here
// instead of on eight lanes of the block's warp).
__global__ void __launch_bounds__(256)
zc1_eq_basis_kernel(const gf128* __restrict__ eq, size_t n, const ZcRound1Tables* __restrict__ T,
                    gf128* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * 8; i += (size_t)gridDim.x * blockDim.x) {
    const uint64_t* f = T->phi8[1u << (i & 7)];
    out[i] = gf_mul(gf128{{(uint32_t)f[0], (uint32_t)(f[0] >> 32), (uint32_t)f[1], (uint32_t)(f[1] >> 32)}},
                    gf_load(&eq[i >> 3]));
  }
}

// XOR-reduce `count` rows of `width` F128 into out: each block owns 8 columns
// and 32 row lanes, then folds the row lanes in shared memory.
__global__ void __launch_bounds__(256)
reduce_rows_kernel(const gf128* __restrict__ in, size_t count, int width, gf128* __restrict__ out) {
  __shared__ gf128 red[32][8];
  const int cl = threadIdx.x & 7, rl = threadIdx.x >> 3;
  const int col = blockIdx.x * 8 + cl;
  gf128 acc = gf_zero();
  if (col < width)
    for (size_t r = rl; r < count; r += 32) acc = gf_add(acc, in[r * width + col]);
  red[rl][cl] = acc;
  __syncthreads();
  if (rl == 0 && col < width) {
    for (int k = 1; k < 32; k++) acc = gf_add(acc, red[k][cl]);
    out[col] = acc;
  }
}

// eq table split: lo[i] = prod_{k<lo_bits} f(r_k, bit k of i), hi[i] over the
// next hi_bits variables; f(r, 1) = r, f(r, 0) = 1 + r. Each CTA first builds
// the eq tables of 7-bit chunks of the variables in shared memory (at most
// 4 x 128 entries per set), so an entry costs (chunks - 1) products instead
// of one per variable.
constexpr int EQ_CHUNK = 7, EQ_MAX_CHUNKS = 4;
// One table pair, CTA `blk` of `nblk` (the calling kernel's grid slice).
__device__ __forceinline__ void eq_split_body(const gf128* __restrict__ r, int lo_bits, int hi_bits,
                                              gf128* __restrict__ lo, gf128* __restrict__ hi, size_t blk,
                                              size_t nblk) {
  __shared__ gf128 t[2][EQ_MAX_CHUNKS][1 << EQ_CHUNK];
  for (int e = threadIdx.x; e < 2 * EQ_MAX_CHUNKS * (1 << EQ_CHUNK); e += blockDim.x) {
    const int set = e / (EQ_MAX_CHUNKS << EQ_CHUNK), c = (e >> EQ_CHUNK) % EQ_MAX_CHUNKS, v = e & ((1 << EQ_CHUNK) - 1);
    const int nb = set ? hi_bits : lo_bits;
    const gf128* rr = (set ? r + lo_bits : r) + EQ_CHUNK * c;
    const int cb = nb - EQ_CHUNK * c < EQ_CHUNK ? nb - EQ_CHUNK * c : EQ_CHUNK;
    if (cb <= 0 || v >= (1 << cb)) continue;
    gf128 acc = gf_one();
    for (int k = 0; k < cb; k++) {
      gf128 rk = rr[k];
      if (!((v >> k) & 1)) rk.w[0] ^= 1;
      acc = gf_mul(acc, rk);
    }
    t[set][c][v] = acc;
  }
  __syncthreads();
  const size_t nlo = (size_t)1 << lo_bits, nhi = (size_t)1 << hi_bits;
  for (size_t e = blk * blockDim.x + threadIdx.x; e < nlo + nhi; e += nblk * blockDim.x) {
    const bool is_lo = e < nlo;
    const size_t idx = is_lo ? e : e - nlo;
    const int set = is_lo ? 0 : 1, nb = is_lo ? lo_bits : hi_bits;
    const int nch = (nb + EQ_CHUNK - 1) / EQ_CHUNK;
    gf128 acc = gf_one();
    for (int c = 0; c < nch; c++) {
      const gf128 f = t[set][c][(idx >> (EQ_CHUNK * c)) & ((1 << EQ_CHUNK) - 1)];
      acc = c == 0 ? f : gf_mul(acc, f);
    }
    if (is_lo) lo[idx] = acc;
    else hi[idx] = acc;
  }
}

__global__ void __launch_bounds__(256)
eq_split_kernel(const gf128* __restrict__ r, int lo_bits, int hi_bits, gf128* __restrict__ lo,
                gf128* __restrict__ hi) {
  eq_split_body(r, lo_bits, hi_bits, lo, hi, blockIdx.x, gridDim.x);
}

// Many table pairs in one launch: job blockIdx.y, its tables split over the
// x dimension.
__global__ void __launch_bounds__(256)
eq_split_multi_kernel(const FlockEqJob* __restrict__ jobs) {
  const FlockEqJob j = jobs[blockIdx.y];
  eq_split_body((const gf128*)j.r, j.lo_bits, j.hi_bits, (gf128*)j.lo, (gf128*)j.hi, blockIdx.x, gridDim.x);
}

// One multilinear round (zerocheck.rs:690-760, multilinear.rs:632-675), with
// the previous round's bind fused in when rho != null:
//   in:  A, B of length 2*n_pairs_in (bound to A' = A0 + rho (A0 + A1) first)
//   msg: G(1) = sum_j eq[j] a1 b1,  G(inf) = sum_j eq[j] (a0+a1)(b0+b1)
// eq[j] = eq_lo[j & lo_mask] * eq_hi[j >> lo_bits]: the inner sums run over
// eq_lo only and are multiplied by eq_hi once per CTA row block.
constexpr int RND_THREADS = 256;
#ifndef ZC_UNROLL
#define ZC_UNROLL 1
#endif
constexpr int kZcUnroll = ZC_UNROLL;
#ifndef ZC_RND_MIN_BLOCKS
#define ZC_RND_MIN_BLOCKS 2  // two resident blocks per SM (128 registers) measured best
#endif
// use_tab: the bind multiplies through rho's byte tables (gf_tab.cuh, dynamic
// shared memory), worth their build when a CTA binds hundreds of pairs.
__global__ void __launch_bounds__(RND_THREADS, ZC_RND_MIN_BLOCKS)
zc_round_kernel(const gf128* __restrict__ A, const gf128* __restrict__ B, size_t n_pairs, int bind,
                const __grid_constant__ gf128p rho, const gf128 rho_plain, int use_tab, gf128* __restrict__ Aout,
                gf128* __restrict__ Bout, const gf128* __restrict__ eq_lo, const gf128* __restrict__ eq_hi,
                int lo_bits, gf128* __restrict__ partials) {
  extern __shared__ uint4 rtab[];
  const uint32_t rot = threadIdx.x & 15;
  if (use_tab) gf_tab_build(rho_plain, rtab);
  // grid-stride over hi blocks: each CTA handles whole hi indices
  const size_t lo_n = (size_t)1 << lo_bits;
  const size_t n_hi = (n_pairs + lo_n - 1) / lo_n;
  gf256 g1 = {{0, 0, 0, 0}}, gi = {{0, 0, 0, 0}};
  for (size_t h = blockIdx.x; h < n_hi; h += gridDim.x) {
    gf256 l1 = {{0, 0, 0, 0}}, li = {{0, 0, 0, 0}};
    size_t base = h * lo_n;
    size_t end = base + lo_n < n_pairs ? base + lo_n : n_pairs;
#pragma unroll kZcUnroll
    for (size_t j = base + threadIdx.x; j < end; j += RND_THREADS) {
      gf128 a0, a1, b0, b1;
      if (bind) {
        gf128 p0 = A[4 * j], p1 = A[4 * j + 1], p2 = A[4 * j + 2], p3 = A[4 * j + 3];
        gf128 q0 = B[4 * j], q1 = B[4 * j + 1], q2 = B[4 * j + 2], q3 = B[4 * j + 3];
        if (use_tab) {
          a0 = gf_add(p0, gf_mul_tab(rtab, gf_add(p0, p1), rot));
          a1 = gf_add(p2, gf_mul_tab(rtab, gf_add(p2, p3), rot));
          b0 = gf_add(q0, gf_mul_tab(rtab, gf_add(q0, q1), rot));
          b1 = gf_add(q2, gf_mul_tab(rtab, gf_add(q2, q3), rot));
        } else {
          a0 = gf_add(p0, gf_mul_p(gf_add(p0, p1), rho));
          a1 = gf_add(p2, gf_mul_p(gf_add(p2, p3), rho));
          b0 = gf_add(q0, gf_mul_p(gf_add(q0, q1), rho));
          b1 = gf_add(q2, gf_mul_p(gf_add(q2, q3), rho));
        }
        Aout[2 * j] = a0; Aout[2 * j + 1] = a1;
        Bout[2 * j] = b0; Bout[2 * j + 1] = b1;
      } else {
        a0 = A[2 * j]; a1 = A[2 * j + 1]; b0 = B[2 * j]; b1 = B[2 * j + 1];
      }
      gf128 e = eq_lo[j - base];
      gf256_acc(l1, gf_mul_wide(e, gf_mul(a1, b1)));
      gf256_acc(li, gf_mul_wide(e, gf_mul(gf_add(a0, a1), gf_add(b0, b1))));
    }
    gf128 eh = eq_hi[h];
    gf256_acc(g1, gf_mul_wide(eh, gf256_reduce(l1)));
    gf256_acc(gi, gf_mul_wide(eh, gf256_reduce(li)));
  }
  // block reduction of the two unreduced sums
  __shared__ gf256 red[2][RND_THREADS / 32];
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      g1.r[k] ^= __shfl_xor_sync(0xffffffffu, g1.r[k], off);
      gi.r[k] ^= __shfl_xor_sync(0xffffffffu, gi.r[k], off);
    }
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][warp] = g1; red[1][warp] = gi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    gf256 s1 = {{0, 0, 0, 0}}, si = {{0, 0, 0, 0}};
    for (int w = 0; w < RND_THREADS / 32; w++) { gf256_acc(s1, red[0][w]); gf256_acc(si, red[1][w]); }
    partials[2 * blockIdx.x] = gf256_reduce(s1);
    partials[2 * blockIdx.x + 1] = gf256_reduce(si);
  }
}

// Round 0 fused with the skip fold: the tables A0, B0 (sum_s bit_s(W[x]) L_s(z),
// eight byte tables of the 64 Lagrange weights) are computed from the bit rows
// of a and b, written for round 1, and used at once for round 0's message
// (G(1), G(inf) as in zc_round_kernel), so A0/B0 are never read back here and
// the table lookups overlap the round's GF(2^128) products.
__global__ void __launch_bounds__(RND_THREADS, ZC_RND_MIN_BLOCKS)
zc_round0_skip_kernel(const uint64_t* __restrict__ W0, const uint64_t* __restrict__ W1, size_t n_pairs,
                      const gf128* __restrict__ lag, gf128* __restrict__ A0, gf128* __restrict__ B0,
                      const gf128* __restrict__ eq_lo, const gf128* __restrict__ eq_hi, int lo_bits,
                      gf128* __restrict__ partials) {
  extern __shared__ gf128 tab[];  // [8][256]
  for (int e = threadIdx.x; e < 8 * 256; e += blockDim.x) {
    int c = e >> 8, v = e & 255;
    gf128 acc = gf_zero();
    for (int j = 0; j < 8; j++)
      if ((v >> j) & 1) acc = gf_add(acc, lag[8 * c + j]);
    tab[e] = acc;
  }
  __syncthreads();
  auto skip = [&](uint64_t w) {
    gf128 r = gf_zero();
#pragma unroll
    for (int c = 0; c < 8; c++) r = gf_add(r, tab[c * 256 + ((w >> (8 * c)) & 255)]);
    return r;
  };
  const size_t lo_n = (size_t)1 << lo_bits;
  const size_t n_hi = (n_pairs + lo_n - 1) / lo_n;
  gf256 g1 = {{0, 0, 0, 0}}, gi = {{0, 0, 0, 0}};
  for (size_t h = blockIdx.x; h < n_hi; h += gridDim.x) {
    gf256 l1 = {{0, 0, 0, 0}}, li = {{0, 0, 0, 0}};
    size_t base = h * lo_n;
    size_t end = base + lo_n < n_pairs ? base + lo_n : n_pairs;
    for (size_t j = base + threadIdx.x; j < end; j += RND_THREADS) {
      const uint64_t x0 = W0[2 * j], x1 = W0[2 * j + 1], y0 = W1[2 * j], y1 = W1[2 * j + 1];
      const gf128 a0 = skip(x0), a1 = skip(x1), b0 = skip(y0), b1 = skip(y1);
      A0[2 * j] = a0; A0[2 * j + 1] = a1;
      B0[2 * j] = b0; B0[2 * j + 1] = b1;
      const gf128 e = eq_lo[j - base];
      gf256_acc(l1, gf_mul_wide(e, gf_mul(a1, b1)));
      gf256_acc(li, gf_mul_wide(e, gf_mul(gf_add(a0, a1), gf_add(b0, b1))));
    }
    const gf128 eh = eq_hi[h];
    gf256_acc(g1, gf_mul_wide(eh, gf256_reduce(l1)));
    gf256_acc(gi, gf_mul_wide(eh, gf256_reduce(li)));
  }
  __shared__ gf256 red[2][RND_THREADS / 32];
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      g1.r[k] ^= __shfl_xor_sync(0xffffffffu, g1.r[k], off);
      gi.r[k] ^= __shfl_xor_sync(0xffffffffu, gi.r[k], off);
    }
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][warp] = g1; red[1][warp] = gi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    gf256 s1 = {{0, 0, 0, 0}}, si = {{0, 0, 0, 0}};
    for (int w = 0; w < RND_THREADS / 32; w++) { gf256_acc(s1, red[0][w]); gf256_acc(si, red[1][w]); }
    partials[2 * blockIdx.x] = gf256_reduce(s1);
    partials[2 * blockIdx.x + 1] = gf256_reduce(si);
  }
}

// Block reduction of two unreduced sums into partials[2 * block], [2 * block + 1].
__device__ __forceinline__ void block_reduce2(gf256 g1, gf256 gi, gf128* __restrict__ partials) {
  __shared__ gf256 red[2][RND_THREADS / 32];
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      g1.r[k] ^= __shfl_xor_sync(0xffffffffu, g1.r[k], off);
      gi.r[k] ^= __shfl_xor_sync(0xffffffffu, gi.r[k], off);
    }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][warp] = g1; red[1][warp] = gi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    gf256 s1 = {{0, 0, 0, 0}}, si = {{0, 0, 0, 0}};
    for (int w = 0; w < RND_THREADS / 32; w++) { gf256_acc(s1, red[0][w]); gf256_acc(si, red[1][w]); }
    partials[2 * blockIdx.x] = gf256_reduce(s1);
    partials[2 * blockIdx.x + 1] = gf256_reduce(si);
  }
}

// Multilinear rounds 0..5, whose lowest eq variables are fixed challenges
// (zerocheck/univariate_skip_optimized.rs:85-130): r7, r8 are phi8 constants
// and r9..r12 are g / (1 + g) with g = x^(2^k), so eq(r_k, b) = (1 + r_k) x^(b 2^k).
// With s = a_bits + m_bits, pair j = h per_h + (g << s) + (jm << a_bits) + ja
// (ja over the phi8 variables, jm over the shift variables, g and h over the
// rest) has eq(j) = eq_lo[(g << a_bits) | ja] x^(m_mul jm) Dinv eq_hi[h], where
// eq_lo / eq_hi are the eq tables of the phi8 and remaining variables and
// Dinv = prod (1 + r_k) over the shift variables (applied on the host). So the
// products a1 b1 and (a0 + a1)(b0 + b1) of an item's 2^m_bits pairs are summed
// as shifted 143-bit XORs and weighted by eq_lo once per item: two GF(2^128)
// products per pair instead of four. SKIP: round 0, the pairs' values come
// from the skip fold of the bit rows (as in zc_round0_skip_kernel) and are
// written to Aout, Bout; otherwise the 2 n_pairs-entry tables in0, in1 are
// bound at rho into Aout, Bout (as in zc_round_kernel).
// The binding rounds multiply every entry pair by rho through rho's byte
// tables (gf_tab.cuh), built once per CTA.
template <bool SKIP>
__global__ void __launch_bounds__(RND_THREADS, ZC_RND_MIN_BLOCKS)
zc_round_grp_kernel(const void* __restrict__ in0, const void* __restrict__ in1, size_t n_pairs,
                    const gf128 rho, const gf128* __restrict__ lag, gf128* __restrict__ Aout,
                    gf128* __restrict__ Bout, const gf128* __restrict__ eq_lo, const gf128* __restrict__ eq_hi,
                    int lo_bits, int a_bits, int m_bits, int m_mul, gf128* __restrict__ partials) {
  // SKIP: [256 v][8 c] subset sums of the Lagrange weights of byte position c;
  // entry (v, c) sits in bank group c and lane l starts at byte position l mod
  // 8, so eight consecutive lanes read eight distinct bank groups.
  // Otherwise: rho's byte tables (a prefetch slot per thread for the next
  // pair, as in the NTT table passes, measured slower here: these rounds are
  // ALU-bound).
  extern __shared__ gf128 tab[];
  uint4* rtab = reinterpret_cast<uint4*>(tab);
  const uint32_t rot = threadIdx.x & 15;
  if constexpr (!SKIP) gf_tab_build(rho, rtab);
  if constexpr (SKIP) {
    for (int e = threadIdx.x; e < 8 * 256; e += blockDim.x) {
      const int v = e >> 3, c = e & 7;
      gf128 acc = gf_zero();
      for (int k = 0; k < 8; k++)
        if ((v >> k) & 1) acc = gf_add(acc, lag[8 * c + k]);
      tab[e] = acc;
    }
    __syncthreads();
  }
  const int lane8 = threadIdx.x & 7;
  auto skip = [&](uint64_t w) {
    gf128 r = gf_zero();
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int c = (lane8 + k) & 7;
      r = gf_add(r, tab[((((uint32_t)(w >> (8 * c))) & 255) << 3) + c]);
    }
    return r;
  };
  const int s = a_bits + m_bits;
  const size_t items = (size_t)1 << lo_bits;
  const size_t per_h = items << m_bits;
  const size_t n_hi = n_pairs / per_h;
  const size_t amask = ((size_t)1 << a_bits) - 1;
  gf256 g1 = {{0, 0, 0, 0}}, gi = {{0, 0, 0, 0}};
  for (size_t h = blockIdx.x; h < n_hi; h += gridDim.x) {
    gf256 l1 = {{0, 0, 0, 0}}, li = {{0, 0, 0, 0}};
    const size_t base = h * per_h;
    for (size_t it = threadIdx.x; it < items; it += RND_THREADS) {
      const size_t j0 = base + ((it >> a_bits) << s) + (it & amask);
      Acc9 t1, ti;
#pragma unroll
      for (int k = 0; k < 9; k++) { t1.w[k] = 0; ti.w[k] = 0; }
      for (int jm = 0; jm < (1 << m_bits); jm++) {
        const size_t j = j0 + ((size_t)jm << a_bits);
        gf128 a0, a1, b0, b1;
        if constexpr (SKIP) {
          const uint64_t* W0 = reinterpret_cast<const uint64_t*>(in0);
          const uint64_t* W1 = reinterpret_cast<const uint64_t*>(in1);
          const uint64_t x0 = W0[2 * j], x1 = W0[2 * j + 1], y0 = W1[2 * j], y1 = W1[2 * j + 1];
          a0 = skip(x0); a1 = skip(x1); b0 = skip(y0); b1 = skip(y1);
        } else {
          const gf128* A = reinterpret_cast<const gf128*>(in0);
          const gf128* B = reinterpret_cast<const gf128*>(in1);
          const gf128 p0 = A[4 * j], p1 = A[4 * j + 1], p2 = A[4 * j + 2], p3 = A[4 * j + 3];
          a0 = gf_add(p0, gf_mul_tab(rtab, gf_add(p0, p1), rot));
          a1 = gf_add(p2, gf_mul_tab(rtab, gf_add(p2, p3), rot));
          const gf128 q0 = B[4 * j], q1 = B[4 * j + 1], q2 = B[4 * j + 2], q3 = B[4 * j + 3];
          b0 = gf_add(q0, gf_mul_tab(rtab, gf_add(q0, q1), rot));
          b1 = gf_add(q2, gf_mul_tab(rtab, gf_add(q2, q3), rot));
        }
        Aout[2 * j] = a0; Aout[2 * j + 1] = a1;
        Bout[2 * j] = b0; Bout[2 * j + 1] = b1;
        const uint32_t sh = (uint32_t)(jm * m_mul);
        acc9_shift_xor(t1, gf_mul_wide(a1, b1), sh);
        acc9_shift_xor(ti, gf_mul_wide(gf_add(a0, a1), gf_add(b0, b1)), sh);
      }
      const gf128 e = eq_lo[it];
      gf256_acc(l1, gf_mul_wide(e, acc9_reduce(t1)));
      gf256_acc(li, gf_mul_wide(e, acc9_reduce(ti)));
    }
    const gf128 eh = eq_hi[h];
    gf256_acc(g1, gf_mul_wide(eh, gf256_reduce(l1)));
    gf256_acc(gi, gf_mul_wide(eh, gf256_reduce(li)));
  }
  block_reduce2(g1, gi, partials);
}

// Final bind of the last round: out[j] = A0 + rho (A0 + A1).
__global__ void bind_pairs_kernel(const gf128* __restrict__ A, const gf128* __restrict__ B, size_t n, gf128 rho,
                                  gf128* __restrict__ Aout, gf128* __restrict__ Bout) {
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    gf128 p0 = A[2 * j], p1 = A[2 * j + 1], q0 = B[2 * j], q1 = B[2 * j + 1];
    Aout[j] = gf_add(p0, gf_mul(rho, gf_add(p0, p1)));
    Bout[j] = gf_add(q0, gf_mul(rho, gf_add(q0, q1)));
  }
}

}  // namespace

int flock_launch_zc_round1(const void* a, const void* b, const void* c, size_t n_outer, const void* eq_basis,
                           const ZcRound1Tables* d_tables, void* partials, int grid, cudaStream_t st) {
  const size_t smem = R1_SMEM;
  flock_once_per_device((const void*)zc_round1_kernel, [] {
    cudaFuncSetAttribute(zc_round1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)R1_SMEM);
  });
  zc_round1_kernel<<<grid, R1_THREADS, smem, st>>>((const uint64_t*)a, (const uint64_t*)b, (const uint64_t*)c,
                                                   n_outer, (const uint4*)eq_basis, d_tables, (gf128*)partials); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}


int flock_launch_zc1_eq_basis(const void* eq_out, size_t n_outer, const ZcRound1Tables* d_tables, void* out,
                              cudaStream_t st) {
  const size_t items = n_outer * 8;
  const unsigned grid = (unsigned)std::min<size_t>((items + 255) / 256, (size_t)152 * 16);
  zc1_eq_basis_kernel<<<grid, 256, 0, st>>>((const gf128*)eq_out, n_outer, d_tables, (gf128*)out);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_reduce_rows(const void* in, size_t count, int width, void* out, cudaStream_t st) {
  reduce_rows_kernel<<<(width + 7) / 8, 256, 0, st>>>((const gf128*)in, count, width, (gf128*)out); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_eq_split_multi(const FlockEqJob* d_jobs, int n_jobs, size_t max_entries, cudaStream_t st) {
  if (n_jobs <= 0) return FLOCK_OK;
  if (n_jobs > 65535) return FLOCK_ERR_SHAPE;
  size_t gx = (max_entries + 2047) / 2048;  // >= 8 entries per thread, as in flock_launch_eq_split
  if (gx < 1) gx = 1;
  if (gx > 152) gx = 152;
  eq_split_multi_kernel<<<dim3((unsigned)gx, (unsigned)n_jobs), 256, 0, st>>>(d_jobs); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_eq_split(const void* r, int lo_bits, int hi_bits, void* lo, void* hi, cudaStream_t st) {
  if (lo_bits < 0 || hi_bits < 0 || lo_bits > EQ_CHUNK * EQ_MAX_CHUNKS || hi_bits > EQ_CHUNK * EQ_MAX_CHUNKS)
    return FLOCK_ERR_SHAPE;
  size_t n = ((size_t)1 << lo_bits) + ((size_t)1 << hi_bits);
  size_t grid = (n + 2047) / 2048;  // >= 8 entries per thread: the chunk tables are built per CTA
  if (grid > 152) grid = 152;
  eq_split_kernel<<<(unsigned)grid, 256, 0, st>>>((const gf128*)r, lo_bits, hi_bits, (gf128*)lo, (gf128*)hi); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_zc_round(const void* A, const void* B, size_t n_pairs, int bind, const uint64_t rho[2],
                          void* Aout, void* Bout, const void* eq_lo, const void* eq_hi, int lo_bits, void* partials,
                          int grid, cudaStream_t st) {
  gf128 r;
  r.w[0] = (uint32_t)rho[0]; r.w[1] = (uint32_t)(rho[0] >> 32); r.w[2] = (uint32_t)rho[1]; r.w[3] = (uint32_t)(rho[1] >> 32);
  constexpr size_t kTabSmem = (size_t)GF_TAB_ENTRIES * 16;
  flock_once_per_device((const void*)zc_round_kernel, [] {
    cudaFuncSetAttribute(zc_round_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTabSmem);
  });
  const int use_tab = bind && n_pairs / (size_t)grid >= 512;
  zc_round_kernel<<<grid, RND_THREADS, use_tab ? kTabSmem : 0, st>>>(
      (const gf128*)A, (const gf128*)B, n_pairs, bind, gf_prepare(r), r, use_tab, (gf128*)Aout, (gf128*)Bout,
      (const gf128*)eq_lo, (const gf128*)eq_hi, lo_bits, (gf128*)partials);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_bind_pairs(const void* A, const void* B, size_t n, const uint64_t rho[2], void* Aout, void* Bout,
                            cudaStream_t st) {
  gf128 r;
  r.w[0] = (uint32_t)rho[0]; r.w[1] = (uint32_t)(rho[0] >> 32); r.w[2] = (uint32_t)rho[1]; r.w[3] = (uint32_t)(rho[1] >> 32);
  size_t grid = (n + 255) / 256;
  if (grid > 152 * 8) grid = 152 * 8;
  bind_pairs_kernel<<<(unsigned)grid, 256, 0, st>>>((const gf128*)A, (const gf128*)B, n, r, (gf128*)Aout,
                                                    (gf128*)Bout); flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_zc_round_grp(const void* in0, const void* in1, size_t n_pairs, int skip, const uint64_t rho[2],
                              const void* lag, void* Aout, void* Bout, const void* eq_lo, const void* eq_hi,
                              int lo_bits, int a_bits, int m_bits, int m_mul, void* partials, int grid,
                              cudaStream_t st) {
  // the item sums of 2^m_bits shifted products must stay below bit 143
  if (a_bits < 0 || a_bits > lo_bits || m_bits < 1 || m_bits > 4 || m_mul < 1 || m_mul * ((1 << m_bits) - 1) > 15)
    return FLOCK_ERR_SHAPE;
  const size_t per_h = ((size_t)1 << lo_bits) << m_bits;
  if (n_pairs % per_h != 0 || grid < 1) return FLOCK_ERR_SHAPE;
  gf128 r;
  r.w[0] = (uint32_t)rho[0]; r.w[1] = (uint32_t)(rho[0] >> 32); r.w[2] = (uint32_t)rho[1]; r.w[3] = (uint32_t)(rho[1] >> 32);
  constexpr size_t kTabSmem = (size_t)GF_TAB_ENTRIES * 16;
  flock_once_per_device((const void*)zc_round_grp_kernel<false>, [] {
    cudaFuncSetAttribute(zc_round_grp_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTabSmem);
  });
  if (skip)
    zc_round_grp_kernel<true><<<grid, RND_THREADS, 8 * 256 * sizeof(gf128), st>>>(
        in0, in1, n_pairs, r, (const gf128*)lag, (gf128*)Aout, (gf128*)Bout, (const gf128*)eq_lo,
        (const gf128*)eq_hi, lo_bits, a_bits, m_bits, m_mul, (gf128*)partials);
  else
    zc_round_grp_kernel<false><<<grid, RND_THREADS, kTabSmem, st>>>(
        in0, in1, n_pairs, r, (const gf128*)lag, (gf128*)Aout, (gf128*)Bout, (const gf128*)eq_lo,
        (const gf128*)eq_hi, lo_bits, a_bits, m_bits, m_mul, (gf128*)partials);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

int flock_launch_zc_round0_skip(const void* a, const void* b, size_t n_pairs, const void* lag, void* A0, void* B0,
                                const void* eq_lo, const void* eq_hi, int lo_bits, void* partials, int grid,
                                cudaStream_t st) {
  zc_round0_skip_kernel<<<grid, RND_THREADS, 8 * 256 * sizeof(gf128), st>>>(
      (const uint64_t*)a, (const uint64_t*)b, n_pairs, (const gf128*)lag, (gf128*)A0, (gf128*)B0,
      (const gf128*)eq_lo, (const gf128*)eq_hi, lo_bits, (gf128*)partials);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

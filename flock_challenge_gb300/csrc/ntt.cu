// Interleaved additive NTT over GF(2^128) (LCH novel basis, neighbours-last).
//
// Restates AdditiveNttF128::forward_transform_interleaved_from_layer
// (crates/flock-core/src/ntt/additive_ntt_f128.rs:599-622, scalar form at
// :1281-1312): data[pos * num_ntts + lane]; at layer l the pair distance is
// 2^(log_d-l-1) positions and block b = pos >> (log_d - l) uses twiddle
// t(l, b) = table[2^l - 1 + b]; butterfly u += v*t, v += u.
//
// GB300 mapping: a pass applies F <= 8 consecutive layers to a tile of 2^F
// positions x 16 lanes (8 when the code has 8 lanes). The tile's positions
// differ only in the F pair bits of those layers, so every butterfly of the
// pass stays in the tile and the pass costs one HBM read and one write of the
// codeword. Each thread holds one lane of 16 positions in registers and
// applies up to four layers there (eight independent GF(2^128) products per
// layer keep the integer pipes busy), then the tile is exchanged once through
// shared memory for the remaining layers. Each tile row (16 lanes x 16 B) is a
// contiguous 256-byte run, read and written with 16-byte vector accesses. A
// pass may read its input from a separate source with a position mask: the
// first pass of a rate-1/2^r code reads the message directly, position p
// taking row p mod 2^(log_d - r), which is the replicated state after the r
// copy layers (pcs/commit.rs:451-473).
#include <cstdio>
#include <cuda.h>

#include <map>
#include <cstdlib>
#include <mutex>
#include <tuple>
#include <vector>

#include "flock_internal.h"
#include "gf128.cuh"
#include "gf_tab.cuh"
#include "host_field.h"

namespace {


// One pass of F layers (l0 .. l0+F-1) over tiles of 2^F positions x TL lanes.
// A thread keeps one lane of 2^E positions (E = min(F, 4)) in registers, so a
// layer gives it 2^(E-1) independent butterflies; the pass runs as two stages
// of at most four layers (the top k1 pair bits, then the low k2 bits) with one
// shared-memory exchange between them. Loads and stores go straight between
// HBM and registers: the TL lanes of a position are a contiguous TL*16-byte run.
// Pass shape variants: positions per thread (log2) and the resident threads
// per SM the register budget is sized for. The autotuner below times them per
// transform shape on the device and keeps the fastest; variant 1 is the
// default when tuning is off.
//   variant 0: 4 positions per thread, 768 threads/SM (passes of <= 4 layers)
//   variant 1: 8 positions per thread, 512 threads/SM (passes of <= 6 layers)
//   variant 2: 16 positions per thread, 256 threads/SM (passes of <= 8 layers)
constexpr int kVariants = 3;
constexpr int kDefaultVariant = 1;
__host__ __device__ constexpr int variant_pos_log(int v) { return v == 0 ? 2 : v == 1 ? 3 : 4; }
__host__ __device__ constexpr int variant_sm_threads(int v) { return v == 0 ? 768 : v == 1 ? 512 : 256; }
__host__ __device__ constexpr int variant_max_layers(int v) {
  return 2 * variant_pos_log(v) < 8 ? 2 * variant_pos_log(v) : 8;
}

template <int F, int TL, int V>
struct PassShape {
  static constexpr int E = F < variant_pos_log(V) ? F : variant_pos_log(V);  // positions per thread (log2)
  static constexpr int K1 = F <= E ? F : (F + 1) / 2 < E ? (F + 1) / 2 : E;  // stage 1 layers
  static constexpr int K2 = F - K1;
  static_assert(K2 <= E, "a pass covers at most twice the positions-per-thread bits");
  static constexpr int PT = 1 << (F - E);            // threads per lane
  static constexpr int THREADS = TL * PT;
  static constexpr int SMEM = K2 > 0 ? (1 << F) * TL * 16 : 16;
  static constexpr int WARP_THREADS = THREADS < 32 ? 32 : THREADS;  // a block occupies whole warps
  static constexpr int BLOCKS_FIT = variant_sm_threads(V) / WARP_THREADS;
  static constexpr int MIN_BLOCKS = BLOCKS_FIT < 1 ? 1 : BLOCKS_FIT > 32 ? 32 : BLOCKS_FIT;
};

// Tile position of the element with label j in stage 1 / stage 2. Labels are
// ordered so that the pair bits of the stage's layers are the label's top bits
// in layer order (stage 1: tile bits F-1 .. F-K1; stage 2: tile bits K2-1 .. 0);
// the other label bits and the thread index pt fill the remaining tile bits.
template <int F, int E, int K1>
__device__ __forceinline__ int pos_stage1(int pt, int j) {
  return ((j >> (E - K1)) << (F - K1)) | (pt << (E - K1)) | (j & ((1 << (E - K1)) - 1));
}
template <int F, int E, int K2>
__device__ __forceinline__ int pos_stage2(int pt, int j) {
  return ((j & ((1 << (E - K2)) - 1)) << (F - (E - K2))) | (pt << K2) | (j >> (E - K2));
}
template <int E>
__host__ __device__ constexpr int rotr_bits(int j, int r) {
  return r == 0 ? j : ((j >> r) | (j << (E - r))) & ((1 << E) - 1);
}

// PREP: the twiddle table holds prepared operands (gf128p) instead of plain
// elements, so the products skip the twiddle's masking.
template <int F, int TL, bool PREP, int V>
__global__ void __launch_bounds__(PassShape<F, TL, V>::THREADS, PassShape<F, TL, V>::MIN_BLOCKS)
ntt_pass_kernel(gf128* __restrict__ dst, const gf128* __restrict__ src, size_t src_pos_mask,
                const void* __restrict__ tw_any, int log_d, int log_lanes, int l0, int narrow) {
  using S = PassShape<F, TL, V>;
  constexpr int E = S::E, K1 = S::K1, K2 = S::K2, NE = 1 << E, H = NE / 2;
  extern __shared__ gf128 tile[];
  const int lane_groups = (1 << log_lanes) / TL;
  const size_t tile_id = blockIdx.x / lane_groups;
  const int lg = blockIdx.x % lane_groups;
  const int lo_bits = log_d - l0 - F;
  const size_t lo = tile_id & (((size_t)1 << lo_bits) - 1);
  const size_t hi = tile_id >> lo_bits;
  const size_t nl = (size_t)1 << log_lanes;
  const int ln = threadIdx.x % TL, pt = threadIdx.x / TL;
  const size_t col = (size_t)lg * TL + ln;
  auto gpos = [&](int i) { return (hi << (log_d - l0)) | ((size_t)i << lo_bits) | lo; };

  gf128 y[NE];
#pragma unroll
  for (int j = 0; j < NE; j++) y[j] = gf_load(&src[(gpos(pos_stage1<F, E, K1>(pt, j)) & src_pos_mask) * nl + col]);

  // One layer per iteration, always pairing labels j and j + H (the top label
  // bit); the labels are then rotated left by one bit so the next layer's pair
  // bit is on top. The body stays small (H products), which keeps the hot loop
  // inside the instruction cache.
#pragma unroll 1
  for (int t = 0; t < F; t++) {
    if (K2 > 0 && t == K1) {
      // stage 1 done: labels are rotated by K1; exchange into stage-2 labels
      __syncwarp();
#pragma unroll
      for (int j = 0; j < NE; j++) tile[pos_stage1<F, E, K1>(pt, rotr_bits<E>(j, K1 % E)) * TL + ln] = y[j];
      __syncthreads();
#pragma unroll
      for (int j = 0; j < NE; j++) y[j] = tile[pos_stage2<F, E, K2>(pt, j) * TL + ln];
    }
    const bool st2 = t >= K1;
    const int r = st2 ? t - K1 : t;
    const size_t twb = (((size_t)1) << (l0 + t)) - 1 + (hi << t);
    int ti[H];
#pragma unroll
    for (int j = 0; j < H; j++) {
      const int jo = ((j >> r) | (j << (E - r))) & (NE - 1);
      const int i0 = st2 ? pos_stage2<F, E, K2>(pt, jo) : pos_stage1<F, E, K1>(pt, jo);
      ti[j] = i0 >> (F - t);
    }
    if constexpr (PREP) {
      // Block 0 of every layer has twiddle 0 (the table's subset sums start
      // at the empty sum; all other blocks are non-zero): its butterflies
      // need no product. Blocks are uniform over a tile, so the test rarely
      // diverges.
      // The deepest layers' twiddles are narrow (layer d-1 below 2^d, layer
      // d-2 below 2^(2d-3)): byte 0 of `narrow` is the first layer whose
      // twiddles fit 32 bits, bytes 1, 2, 3 those for 40, 64 and 72 bits (the
      // host reads the bounds off the table). Their products take four (32
      // bits) or six (64 bits) 32-bit products instead of nine; 40 and 72 bits
      // take those of their low 32 or 64 bits plus one shifted copy of the
      // operand per higher set bit. The class is uniform over a layer.
      const gf128p* twl = reinterpret_cast<const gf128p*>(tw_any) + twb;
      const bool hi0 = hi == 0;
      const int layer = l0 + t;
      const int wcls = layer >= (narrow & 255)           ? 1
                       : layer >= ((narrow >> 8) & 255)  ? 4
                       : layer >= ((narrow >> 16) & 255) ? 2
                       : layer >= ((narrow >> 24) & 255) ? 3
                                                         : 0;
      if (wcls == 1) {
#pragma unroll
        for (int j = 0; j < H; j++) {
          if (!(hi0 && ti[j] == 0)) y[j] = gf_add(y[j], gf_mul_p32(y[j + H], twl[ti[j]].m[0]));
          y[j + H] = gf_add(y[j + H], y[j]);
        }
      } else if (wcls == 2) {
#pragma unroll
        for (int j = 0; j < H; j++) {
          if (!(hi0 && ti[j] == 0)) {
            const gf128p* q = &twl[ti[j]];
            y[j] = gf_add(y[j], gf_mul_p64(y[j + H], q->m[0], q->m[1], q->m[2]));
          }
          y[j + H] = gf_add(y[j + H], y[j]);
        }
      } else if (wcls == 4) {
#pragma unroll
        for (int j = 0; j < H; j++) {
          if (!(hi0 && ti[j] == 0)) {
            const gf128p* q = &twl[ti[j]];
            const uint4 m1 = q->m[1];  // word 1 of the twiddle in its four masked parts
            y[j] = gf_add(y[j], gf_mul_p40(y[j + H], q->m[0], m1.x | m1.y | m1.z | m1.w));
          }
          y[j + H] = gf_add(y[j + H], y[j]);
        }
      } else if (wcls == 3) {
#pragma unroll
        for (int j = 0; j < H; j++) {
          if (!(hi0 && ti[j] == 0)) {
            const gf128p* q = &twl[ti[j]];
            const uint4 m3 = q->m[3];  // word 2 of the twiddle in its four masked parts
            y[j] = gf_add(y[j], gf_mul_p72(y[j + H], q->m[0], q->m[1], q->m[2], m3.x | m3.y | m3.z | m3.w));
          }
          y[j + H] = gf_add(y[j + H], y[j]);
        }
      } else {
#pragma unroll
        for (int j = 0; j < H; j++) {
          if (!(hi0 && ti[j] == 0)) y[j] = gf_add(y[j], gf_mul_p(y[j + H], gf_load_p(&twl[ti[j]])));
          y[j + H] = gf_add(y[j + H], y[j]);
        }
      }
    } else {
      const gf128* twl = reinterpret_cast<const gf128*>(tw_any) + twb;
      gf128 tv[H];
#pragma unroll
      for (int j = 0; j < H; j++) tv[j] = gf_load(&twl[ti[j]]);
#pragma unroll
      for (int j = 0; j < H; j++) {
        y[j] = gf_add(y[j], gf_mul(y[j + H], tv[j]));
        y[j + H] = gf_add(y[j + H], y[j]);
      }
    }
    // rotate labels left by one: new[k] = old[rotr(k, 1)]
    gf128 z[NE];
#pragma unroll
    for (int k = 0; k < NE; k++) z[k] = y[rotr_bits<E>(k, 1 % E)];
#pragma unroll
    for (int k = 0; k < NE; k++) y[k] = z[k];
  }
  if (K2 > 0) {
#pragma unroll
    for (int j = 0; j < NE; j++)
      gf_store(&dst[gpos(pos_stage2<F, E, K2>(pt, rotr_bits<E>(j, K2 % E))) * nl + col], y[j]);
  } else {
#pragma unroll
    for (int j = 0; j < NE; j++)
      gf_store(&dst[gpos(pos_stage1<F, E, K1>(pt, rotr_bits<E>(j, K1 % E))) * nl + col], y[j]);
  }
}

// Twiddle table of the standard basis {1, x, ..., x^(d-1)}:
// normalized subspace-polynomial evaluations (additive_ntt_f128.rs:57-88),
// expanded breadth-first (additive_ntt_f128.rs:106-129).
// Generator rows of the twiddle table: layer l's twiddles are the subset sums
// of rows[d - l - 1][1 .. l].
std::vector<std::vector<hf::F>> twiddle_rows(int d) {
  std::vector<std::vector<hf::F>> ev(d);
  for (int i = 0; i < d; i++) ev[0].push_back(i < 64 ? hf::F(1ULL << i, 0) : hf::F(0, 1ULL << (i - 64)));
  for (int i = 1; i < d; i++)
    for (size_t k = 1; k < ev[i - 1].size(); k++) ev[i].push_back(ev[i - 1][k] * (ev[i - 1][k] + ev[i - 1][0]));
  for (auto& row : ev) {
    hf::F iv = hf::inv(row[0]);
    for (auto& v : row) v = v * iv;
  }
  return ev;
}

std::vector<hf::F> host_twiddles(int d) {
  const std::vector<std::vector<hf::F>> ev = twiddle_rows(d);
  std::vector<hf::F> tw;
  tw.reserve(((size_t)1 << d) - 1);
  for (int layer = 0; layer < d; layer++) {
    size_t start = tw.size();
    const auto& row = ev[d - layer - 1];
    tw.push_back(hf::F());
    for (size_t bit = 0; bit + 1 < row.size(); bit++) {
      size_t half = (size_t)1 << bit;
      for (size_t b = 0; b < half; b++) tw.push_back(tw[start + b] + row[bit + 1]);
    }
  }
  return tw;
}

std::mutex g_tw_mu;
std::map<std::pair<int, int>, void*> g_tw;  // (device, log_d) -> device table

// Bit width of every twiddle of layer `layer` of a 2^log_d transform (the OR of
// the layer's generators bounds all its subset sums), cached per log_d.
int twiddle_layer_width(int log_d, int layer) {
  static std::mutex mu;
  static std::map<int, std::vector<int>> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(log_d);
  if (it == cache.end()) {
    const std::vector<std::vector<hf::F>> ev = twiddle_rows(log_d);
    std::vector<int> w(log_d, 0);
    for (int l = 0; l < log_d; l++) {
      uint64_t lo = 0, hi = 0;
      const auto& row = ev[log_d - l - 1];
      for (int bit = 0; bit < l; bit++) {
        lo |= row[bit + 1].lo;
        hi |= row[bit + 1].hi;
      }
      w[l] = hi ? 128 - __builtin_clzll(hi) : lo ? 64 - __builtin_clzll(lo) : 0;
    }
    it = cache.emplace(log_d, std::move(w)).first;
  }
  return it->second[layer];
}

// w32 | (w40 << 8) | (w64 << 16) | (w72 << 24): the first layers from which
// every twiddle of a transform of 2^log_d positions is below 2^32, 2^40,
// 2^64 and 2^72, read off the table (the normalized subspace polynomials of
// the deepest layers have low degree: layer d-1 below 2^d, layer d-2 below
// 2^(2d-3), layer d-3 below 2^69 at d = 20). Cached per log_d.
constexpr int kMaxTwiddleClassLogD = 40;
int flock_ntt_narrow_layers(int log_d) {
  static std::mutex mu;
  static std::map<int, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(log_d);
  if (it != cache.end()) return it->second;
  // the first layer from which every deeper layer's twiddles fit `bits`
  auto first_fit = [log_d](int bits) {
    int w = log_d;
    while (w > 0 && twiddle_layer_width(log_d, w - 1) <= bits) w--;
    return w;
  };
  return cache[log_d] = first_fit(32) | (first_fit(40) << 8) | (first_fit(64) << 16) | (first_fit(72) << 24);
}

template <int F, bool PREP, int V>
int launch_pass(gf128* dst, const gf128* src, size_t mask, const void* tw, int log_d, int log_lanes, int l0,
                cudaStream_t st) {
  const int narrow = PREP ? flock_ntt_narrow_layers(log_d) : log_d * 0x01010101;
  if constexpr (F > variant_max_layers(V)) {
    return FLOCK_ERR_SHAPE;
  } else {
    size_t tiles = (size_t)1 << (log_d - F);
    if constexpr (PassShape<F, 16, V>::THREADS < 32) {
      // A pass no deeper than the shape's positions per thread needs one
      // thread per lane: with 16 lanes a block would fill half a warp, so
      // codes of 32 lanes or more take 32 lanes per block.
      if (log_lanes >= 5) {
        using S = PassShape<F, 32, V>;
        static_assert(S::SMEM <= 48 * 1024, "one-stage passes use no tile");
        size_t blocks = tiles * ((1 << log_lanes) / 32);
        ntt_pass_kernel<F, 32, PREP, V>
            <<<(unsigned)blocks, S::THREADS, S::SMEM, st>>>(dst, src, mask, tw, log_d, log_lanes, l0, narrow);
        flock_count_launch();
        return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
      }
    }
    if (log_lanes >= 4) {
      using S = PassShape<F, 16, V>;
      size_t blocks = tiles * ((1 << log_lanes) / 16);
      if constexpr (S::SMEM > 48 * 1024) {
        flock_once_per_device((const void*)ntt_pass_kernel<F, 16, PREP, V>, [] {
          cudaFuncSetAttribute(ntt_pass_kernel<F, 16, PREP, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               PassShape<F, 16, V>::SMEM);
        });
      }
      ntt_pass_kernel<F, 16, PREP, V>
          <<<(unsigned)blocks, S::THREADS, S::SMEM, st>>>(dst, src, mask, tw, log_d, log_lanes, l0, narrow);
    } else {
      using S = PassShape<F, 8, V>;
      size_t blocks = tiles * ((1 << log_lanes) / 8);
      ntt_pass_kernel<F, 8, PREP, V>
          <<<(unsigned)blocks, S::THREADS, S::SMEM, st>>>(dst, src, mask, tw, log_d, log_lanes, l0, narrow);
    }
    flock_count_launch();
    return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
  }
}

template <bool PREP, int V>
int run_pass_v(int f, gf128* dst, const gf128* src, size_t mask, const void* tw, int log_d, int log_lanes, int l0,
               cudaStream_t st) {
  switch (f) {
    case 1: return launch_pass<1, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    case 2: return launch_pass<2, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    case 3: return launch_pass<3, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    case 4: return launch_pass<4, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    case 5: return launch_pass<5, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    case 6: return launch_pass<6, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    case 7: return launch_pass<7, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    case 8: return launch_pass<8, PREP, V>(dst, src, mask, tw, log_d, log_lanes, l0, st);
    default: return FLOCK_ERR_SHAPE;
  }
}

// The passes of layers [start_layer, log_d) with variant v: passes of at most
// variant_max_layers(v) layers, split evenly. The first pass reads src with
// the position mask; later passes work in place on dst.
template <bool PREP>
int run_passes(int v, gf128* dst, const gf128* src, size_t mask, const void* tw, int log_d, int log_lanes,
               int start_layer, cudaStream_t st) {
  const int max_f = variant_max_layers(v);
  const int remaining = log_d - start_layer;
  const int passes = (remaining + max_f - 1) / max_f;
  int l = start_layer;
  for (int q = 0; q < passes; q++) {
    const int f = (remaining - (l - start_layer) + (passes - q) - 1) / (passes - q);
    int rc = v == 0 ? run_pass_v<PREP, 0>(f, dst, src, mask, tw, log_d, log_lanes, l, st)
           : v == 1 ? run_pass_v<PREP, 1>(f, dst, src, mask, tw, log_d, log_lanes, l, st)
                    : run_pass_v<PREP, 2>(f, dst, src, mask, tw, log_d, log_lanes, l, st);
    if (rc != FLOCK_OK) return rc;
    src = dst;
    mask = ~(size_t)0;
    l += f;
  }
  return FLOCK_OK;
}

// Plain-twiddle pass of the default shape (the no-allocation entry point).
int run_pass(int f, gf128* dst, const gf128* src, size_t mask, const gf128* tw, int log_d, int log_lanes, int l0,
             cudaStream_t st) {
  return run_pass_v<false, kDefaultVariant>(f, dst, src, mask, tw, log_d, log_lanes, l0, st);
}
constexpr int kMaxPassLayers = variant_max_layers(kDefaultVariant);

// ---- table passes --------------------------------------------------------
//
// In the upper layers a twiddle multiplies many elements: layer l has 2^l
// twiddles, each shared by the 2^(log_d - l - 1) butterflies of its block in
// every lane. Multiplication by a fixed t is GF(2)-linear, so a CTA builds
// byte tables T[(v << 4) + k] = t * v * x^(8k) (16 byte positions k, 256
// values v, 64 KiB) once and then needs 16 table lookups per product instead
// of a carry-less multiply: the products run on the load/store and ALU pipes
// at about twice the rate. A table pass applies layers l and l + 1 to one
// block of layer l (three twiddles: t_A = tw[2^l - 1 + hi] for layer l and
// t_B, t_C for the two halves at layer l + 1); each thread owns a quad of
// positions of one lane.
constexpr int TAB_THREADS = 512;
constexpr int TAB_ENTRIES = GF_TAB_ENTRIES;
constexpr size_t TAB_SMEM = (size_t)3 * TAB_ENTRIES * 16;  // three byte tables
static_assert(TAB_SMEM <= 232448, "table pass shared memory above the 227 KB per-block limit");


// Byte tables of the three twiddles t[0..2] into T (3 x TAB_ENTRIES slots),
// one row (256 per table) per item, computed directly (gf_tab_row_direct):
// every thread works from the start, with no serial nibble phase.
__device__ void build_tabs3(const gf128 t[3], uint4* __restrict__ T) {
  for (int it = threadIdx.x; it < 3 * 256; it += blockDim.x) {
    const int w = it >> 8;
    gf_tab_row_direct(w == 0 ? t[0] : w == 1 ? t[1] : t[2], T + w * TAB_ENTRIES, it & 255);
  }
}

// Layers l, l + 1 of the transform for block hi of layer l (blockIdx.x / cph)
// in all lanes; the cph CTAs of a block split its quads. Position p of a quad:
// (hi << (lo_bits + 2)) | (b << lo_bits) | lo, b = 2-bit quad index.
__global__ void __launch_bounds__(TAB_THREADS, 1)
ntt_tab2_kernel(gf128* __restrict__ dst, const gf128* __restrict__ src, size_t src_pos_mask,
                const gf128* __restrict__ tw, int log_d, int log_lanes, int l, int cph) {
  extern __shared__ uint4 tabs[];  // [3][TAB_ENTRIES]
  const size_t hi = blockIdx.x / cph;
  const int part = blockIdx.x % cph;
  const gf128 t3[3] = {tw[((size_t)1 << l) - 1 + hi], tw[((size_t)1 << (l + 1)) - 1 + 2 * hi],
                       tw[((size_t)1 << (l + 1)) - 1 + 2 * hi + 1]};
  build_tabs3(t3, tabs);
  __syncthreads();
  // block 0 of every layer has twiddle 0: its butterflies need no product
  const bool za = hi == 0, zb = hi == 0;
  const int lo_bits = log_d - l - 2;
  const size_t nl = (size_t)1 << log_lanes;
  const size_t items = ((size_t)1 << lo_bits) << log_lanes;
  const uint32_t rot = threadIdx.x & 15;
  // The next quad is loaded into registers while the current one is computed:
  // with three 64 KiB tables an SM holds 16 warps, too few to hide the global
  // load latency otherwise (measured 1% faster than staging the quad through
  // shared memory with cp.async, whose 32 bytes of shared traffic per element
  // compete with the table lookups). Each quad is read and written by one
  // thread only, so the prefetch is safe in place (dst == src).
  const size_t stride = (size_t)cph * TAB_THREADS;
  size_t it = (size_t)part * TAB_THREADS + threadIdx.x;
  uint4 nx[4];
  auto prefetch = [&](size_t it2) {
    const size_t lane2 = it2 & (nl - 1), lo2 = it2 >> log_lanes;
    const size_t q0 = (hi << (lo_bits + 2)) | lo2;
#pragma unroll
    for (int b = 0; b < 4; b++)
      nx[b] = *reinterpret_cast<const uint4*>(&src[((q0 | ((size_t)b << lo_bits)) & src_pos_mask) * nl + lane2]);
  };
  if (it < items) prefetch(it);
  for (; it < items; it += stride) {
    const size_t lane = it & (nl - 1), lo = it >> log_lanes;
    const size_t p0 = (hi << (lo_bits + 2)) | lo;
    gf128 y[4];
#pragma unroll
    for (int b = 0; b < 4; b++) y[b] = gf128{{nx[b].x, nx[b].y, nx[b].z, nx[b].w}};
    if (it + stride < items) prefetch(it + stride);
    // layer l: pairs (b, b + 2) with t_A
    if (!za) {
      y[0] = gf_add(y[0], gf_mul_tab(tabs, y[2], rot));
      y[1] = gf_add(y[1], gf_mul_tab(tabs, y[3], rot));
    }
    y[2] = gf_add(y[2], y[0]);
    y[3] = gf_add(y[3], y[1]);
    // layer l + 1: pairs (0, 1) with t_B, (2, 3) with t_C
    if (!zb) y[0] = gf_add(y[0], gf_mul_tab(tabs + TAB_ENTRIES, y[1], rot));
    y[1] = gf_add(y[1], y[0]);
    y[2] = gf_add(y[2], gf_mul_tab(tabs + 2 * TAB_ENTRIES, y[3], rot));
    y[3] = gf_add(y[3], y[2]);
#pragma unroll
    for (int b = 0; b < 4; b++) gf_store(&dst[(p0 | ((size_t)b << lo_bits)) * nl + lane], y[b]);
  }
}

// Layers [start, end) handled by table passes: pairs of layers while a block
// of the pass's first layer l holds at least 2^min_log quad-lanes (its three
// tables are then built for at least 4 x 2^min_log products; deeper blocks are
// left to the multiply passes). The autotuner picks min_log per transform
// shape among kTabMinLogs; the default, for untuned calls, is kTabMinLog
// (measured at 2^20 positions x 64 lanes: 2^9 beats 2^11 by 0.3 ms, 2^8 ties
// and 2^7, a lone last layer in the multiply pass, loses 2.2 ms).
constexpr int kTabMinLog = 9;
constexpr int kTabMinLogs[] = {8, 9, 10};
int tab_layers_end(int log_d, int log_lanes, int start, int min_log = kTabMinLog) {
  int l = start;
  while (l + 1 < log_d && log_d - l - 2 + log_lanes >= min_log) l += 2;
  return l;
}

int launch_tab2(gf128* dst, const gf128* src, size_t mask, const gf128* tw, int log_d, int log_lanes, int l,
                cudaStream_t st) {
  flock_once_per_device((const void*)ntt_tab2_kernel, [] {
    cudaFuncSetAttribute(ntt_tab2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAB_SMEM);
  });
  const size_t n_hi = (size_t)1 << l;
  const size_t items = ((size_t)1 << (log_d - l - 2)) << log_lanes;
  // CTAs per block (one resident CTA per SM): minimise waves x per-CTA time,
  // a CTA costing its table build (about 700 products) plus its share of the
  // block's 4 products per quad-lane, with at least one item per thread
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 152;
  // (at least two waves where the block sizes allow: measured faster than one
  // wave of twice-as-long CTAs)
  size_t cph = 1;
  double best = 1e300;
  for (size_t c : {1, 2, 4, 8, 16, 19, 32, 38, 64, 76, 128, 152, 256, 304, 512}) {
    if (c > 1 && items / c < TAB_THREADS) continue;
    if (n_hi * c < 2 * (size_t)sms && items / (2 * c) >= TAB_THREADS) continue;
    const double waves = (double)((n_hi * c + sms - 1) / sms);
    const double t = waves * (700.0 + 4.0 * (double)items / (double)c);
    if (t < best) {
      best = t;
      cph = c;
    }
  }
  ntt_tab2_kernel<<<(unsigned)(n_hi * cph), TAB_THREADS, TAB_SMEM, st>>>(dst, src, mask, tw, log_d, log_lanes, l,
                                                                         (int)cph);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

// ---- deep-table pass ------------------------------------------------------
//
// The twiddles of the last three layers are narrow (layer d-1 below 2^d,
// d-2 below 2^(2d-3), d-3 below 2^69 at d = 20), so a twiddle's carry-less
// products with all 256 byte values fit a small table of unreduced words,
// T[v] = t v: one word for layer d-1, three for d-3. A product y t is then the
// XOR of T[byte k of y] x^(8k) over the 16 bytes of y, reduced once: 16
// lookups instead of four to six 32x32 carry-less pieces. A block owns one
// group of 8 positions in all 64 lanes (a thread per lane): it builds the
// 1 + 4 tables of the group's twiddles for layers d-3 and d-1 (8.25 KiB) and
// applies the three layers to each lane's 8 positions in registers; layer d-2
// keeps the carry-less product of its prepared twiddle (gf_mul_p40), which
// spreads the pass over the ALU and the shared-memory pipes (tables for all
// three layers measured 6.29 ms for the 2^20-position L0 set, this split
// 6.07, the multiply passes 6.65: the random lookups conflict on ~60% of
// shared wavefronts, so the load/store data path binds the all-table form).
// Used for the last three layers of a 64-lane code whose twiddles there fit
// 88, 56 and 24 bits, when the autotuner measures it faster than the
// multiply passes.
constexpr int kDeepVariant = 3;
constexpr int D3_LANES = 64;
constexpr int D3_C_STRIDE = 256 + 16;  // words per layer d-1 table: the skew keeps the build's stores conflict-free

struct Deep3Tabs {
  uint4 a[256];                // layer d-3: t v below 2^96 (three words used)
  uint32_t c[4][D3_C_STRIDE];  // layer d-1, twiddles of the four pairs: below 2^32
};

// The deep-table pass applies to the layers [from, log_d) of a code of
// 2^log_lanes lanes.
bool deep3_applies(int log_d, int log_lanes, int from) {
  return log_d >= 4 && log_d <= 30 && from == log_d - 3 && (1 << log_lanes) == D3_LANES &&
         twiddle_layer_width(log_d, log_d - 1) <= 24 && twiddle_layer_width(log_d, log_d - 2) <= 56 &&
         twiddle_layer_width(log_d, log_d - 3) <= 88;
}

__host__ __device__ constexpr int d3_ctz(int j) { return (j & 1) ? 0 : (j & 2) ? 1 : (j & 4) ? 2 : 3; }

// Words 0..W-1 of a table entry.
__device__ __forceinline__ void d3_words(uint32_t e, uint32_t (&w)[1]) { w[0] = e; }
__device__ __forceinline__ void d3_words(uint4 e, uint32_t (&w)[3]) { w[0] = e.x; w[1] = e.y; w[2] = e.z; }

// y t from the table T[v] = t v of W-word entries. Byte k of y adds T[byte]
// at bit 8k: the lookups go into four accumulators by k mod 4 at word k / 4,
// which are joined once with 8-, 16- and 24-bit funnel shifts (at most
// 128 + 32 W bits), then reduced.
template <int W, class E>
__device__ __forceinline__ gf128 d3_mul(const E* __restrict__ T, const gf128& y) {
  uint32_t acc[4][3 + W];
#pragma unroll
  for (int s = 0; s < 4; s++)
#pragma unroll
    for (int i = 0; i < 3 + W; i++) acc[s][i] = 0;
#pragma unroll
  for (int k = 0; k < 16; k++) {
    const uint32_t v = __byte_perm(y.w[k >> 2], 0, 0x4440u | (uint32_t)(k & 3));
    uint32_t e[W];
    d3_words(T[v], e);
#pragma unroll
    for (int i = 0; i < W; i++) acc[k & 3][(k >> 2) + i] ^= e[i];
  }
  uint32_t r[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    uint32_t x = i < 3 + W ? acc[0][i] : 0u;
#pragma unroll
    for (int s = 1; s < 4; s++) {
      const uint32_t hi = i < 3 + W ? acc[s][i] : 0u, lo = i >= 1 && i - 1 < 3 + W ? acc[s][i - 1] : 0u;
      x ^= __funnelshift_l(lo, hi, 8 * s);
    }
    r[i] = x;
  }
  return gf_reduce(r[0] | ((uint64_t)r[1] << 32), r[2] | ((uint64_t)r[3] << 32), r[4] | ((uint64_t)r[5] << 32),
                   r[6] | ((uint64_t)r[7] << 32));
}

// Layers log_d-3 .. log_d-1 in place for position group blockIdx.x
// (positions 8 q .. 8 q + 7), thread = lane. tw: the plain twiddle table;
// twq: the prepared one (layer d-2's products).
__global__ void __launch_bounds__(D3_LANES, 8) ntt_deep3_kernel(gf128* __restrict__ data, const gf128* __restrict__ tw,
                                                             const gf128p* __restrict__ twq, int log_d) {
  __shared__ Deep3Tabs T;
  const size_t q = blockIdx.x;
  const int lane = threadIdx.x;
  const size_t i17 = ((size_t)1 << (log_d - 3)) - 1 + q;
  const size_t i18 = ((size_t)1 << (log_d - 2)) - 1 + 2 * q;
  const size_t i19 = ((size_t)1 << (log_d - 1)) - 1 + 4 * q;
  // Tables. Thread `lane` owns the entries whose low bits are its index and
  // walks the high bits in Gray order, one XOR per entry; consecutive lanes
  // store consecutive entries.
  {
    // layer d-1: table lane >> 4, entries (j << 4) | (lane & 15)
    const int tb = lane >> 4, lo = lane & 15;
    const uint32_t t = tw[i19 + tb].w[0];
    uint32_t v = 0;
#pragma unroll
    for (int b = 0; b < 4; b++) v ^= (t << b) & (0u - (uint32_t)((lo >> b) & 1));
#pragma unroll
    for (int jj = 0; jj < 16; jj++) {
      if (jj) v ^= t << (4 + d3_ctz(jj));
      T.c[tb][((jj ^ (jj >> 1)) << 4) | lo] = v;
    }
  }
  {
    // layer d-3: entries (j << 6) | lane, three words
    const gf128 t = tw[i17];
    uint32_t v0 = 0, v1 = 0, v2 = 0;
#pragma unroll
    for (int b = 0; b < 6; b++) {
      const uint32_t m = 0u - (uint32_t)((lane >> b) & 1);
      v0 ^= (t.w[0] << b) & m;
      v1 ^= __funnelshift_l(t.w[0], t.w[1], b) & m;
      v2 ^= __funnelshift_l(t.w[1], t.w[2], b) & m;
    }
#pragma unroll
    for (int jj = 0; jj < 4; jj++) {
      if (jj) {
        const int s = 6 + d3_ctz(jj);
        v0 ^= t.w[0] << s;
        v1 ^= __funnelshift_l(t.w[0], t.w[1], s);
        v2 ^= __funnelshift_l(t.w[1], t.w[2], s);
      }
      T.a[((jj ^ (jj >> 1)) << 6) | lane] = make_uint4(v0, v1, v2, 0u);
    }
  }
  __syncthreads();
  gf128 y[8];
#pragma unroll
  for (int j = 0; j < 8; j++) y[j] = gf_load(&data[((q << 3) | (size_t)j) * D3_LANES + lane]);
  // layer d-3: pairs (j, j + 4), one twiddle
#pragma unroll
  for (int j = 0; j < 4; j++) {
    y[j] = gf_add(y[j], d3_mul<3>(T.a, y[j + 4]));
    y[j + 4] = gf_add(y[j + 4], y[j]);
  }
  // layer d-2: pairs (j, j + 2) in each half h, the prepared twiddle of half h
  // (below 2^56: its low word's four masked parts, then one shifted copy of
  // y per set bit of its high word)
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const gf128p* qq = &twq[i18 + h];
    const uint4 m0 = qq->m[0], m1 = qq->m[1];
    const uint32_t thi = m1.x | m1.y | m1.z | m1.w;
#pragma unroll
    for (int j = 4 * h; j < 4 * h + 2; j++) {
      y[j] = gf_add(y[j], gf_mul_p40(y[j + 2], m0, thi));
      y[j + 2] = gf_add(y[j + 2], y[j]);
    }
  }
  // layer d-1: pairs (2 i, 2 i + 1), twiddle c[i]
#pragma unroll
  for (int i = 0; i < 4; i++) {
    y[2 * i] = gf_add(y[2 * i], d3_mul<1>(T.c[i], y[2 * i + 1]));
    y[2 * i + 1] = gf_add(y[2 * i + 1], y[2 * i]);
  }
#pragma unroll
  for (int j = 0; j < 8; j++) gf_store(&data[((q << 3) | (size_t)j) * D3_LANES + lane], y[j]);
}

// The deep-table pass in place on data (the caller checked deep3_applies).
int run_deep3(gf128* data, const gf128* twp, const void* twq, int log_d, cudaStream_t st) {
  ntt_deep3_kernel<<<(unsigned)((size_t)1 << (log_d - 3)), D3_LANES, 0, st>>>(data, twp, (const gf128p*)twq, log_d);
  flock_count_launch();
  return cudaGetLastError() == cudaSuccess ? FLOCK_OK : FLOCK_ERR_CUDA;
}

__global__ void prepare_twiddles_kernel(const gf128* __restrict__ tw, size_t n, gf128p* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = gf_prepare(tw[i]);
}

std::map<std::pair<int, int>, void*> g_twp;  // (device, log_d) -> prepared table (under g_tw_mu)

}  // namespace

const void* flock_ntt_twiddles(int log_d) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto key = std::make_pair(dev, log_d);
  auto it = g_tw.find(key);
  if (it != g_tw.end()) return it->second;
  std::vector<hf::F> tw = host_twiddles(log_d);
  void* d = nullptr;
  if (cudaMalloc(&d, tw.size() * 16 + 16) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, tw.data(), tw.size() * 16, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  g_tw[key] = d;
  return d;
}

// Prepared twiddle table (gf128p per entry), built on the device from the
// plain table once per (device, log_d).
const void* flock_ntt_twiddles_prepared(int log_d) {
  const gf128* tw = (const gf128*)flock_ntt_twiddles(log_d);
  if (!tw) return nullptr;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto key = std::make_pair(dev, log_d);
  auto it = g_twp.find(key);
  if (it != g_twp.end()) return it->second;
  const size_t n = ((size_t)1 << log_d) - 1;
  void* d = nullptr;
  if (cudaMalloc(&d, (n + 1) * sizeof(gf128p)) != cudaSuccess) return nullptr;
  prepare_twiddles_kernel<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256>>>(tw, n, (gf128p*)d);
  flock_count_launch();
  if (cudaDeviceSynchronize() != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  g_twp[key] = d;
  return d;
}

// ---- autotuner -------------------------------------------------------------
//
// Per (device, log_d, lanes, start layer), the first call times on a scratch
// buffer of the same shape (CUDA events on the caller's stream, one warm-up
// and two timed runs per candidate): the table passes for each table depth of
// kTabMinLogs, and the multiply passes of every pass shape from each depth's
// end layer, plus the deep-table pass where a depth leaves exactly the last
// three layers of a 64-lane code; it keeps the pair with the smallest sum for
// later calls. All candidates compute identical results; only speed differs.
// FLOCK_NTT_TUNE=0 in the environment turns tuning off (the default depth and
// shape everywhere); FLOCK_NTT_VARIANT=0|1|2|3 fixes the multiply-pass shape
// (with the default depth; 3 falls back to shape 1 where the deep-table pass
// does not apply).
namespace {

struct TuneKey {
  int dev, log_d, log_lanes, start;
  bool operator<(const TuneKey& o) const {
    return std::tie(dev, log_d, log_lanes, start) < std::tie(o.dev, o.log_d, o.log_lanes, o.start);
  }
};
struct TunedShape {
  int tab_end;  // table passes cover layers [start, tab_end)
  int variant;  // multiply-pass shape of the layers [tab_end, log_d)
};
std::mutex g_tune_mu;
std::map<TuneKey, TunedShape> g_tuned;

bool tuning_enabled() {
  const char* e = std::getenv("FLOCK_NTT_TUNE");
  return !(e && e[0] == '0');
}

// Table passes of layers [from, to) in place on d.
int run_tab_passes(gf128* d, const gf128* twp, int log_d, int log_lanes, int from, int to, cudaStream_t st) {
  for (int l = from; l + 2 <= to; l += 2) {
    const int rc = launch_tab2(d, d, ~(size_t)0, twp, log_d, log_lanes, l, st);
    if (rc != FLOCK_OK) return rc;
  }
  return FLOCK_OK;
}

TunedShape tune_shape(const TuneKey& k, const void* tw, const gf128* twp, cudaStream_t st) {
  TunedShape best{tab_layers_end(k.log_d, k.log_lanes, k.start), kDefaultVariant};
  const size_t bytes = ((size_t)16 << k.log_lanes) << k.log_d;
  void* scratch = nullptr;
  if (cudaMalloc(&scratch, bytes) != cudaSuccess) {
    cudaGetLastError();
    return best;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  gf128* d = (gf128*)scratch;
  cudaMemsetAsync(scratch, 0, bytes, st);
  // ms of fn over two runs after a warm-up one; infinity when a launch fails
  auto time_of = [&](auto&& fn) {
    if (fn() != FLOCK_OK) return 1e30f;
    cudaEventRecord(e0, st);
    bool ok = fn() == FLOCK_OK && fn() == FLOCK_OK;
    cudaEventRecord(e1, st);
    float ms = 0;
    if (!ok || cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      return 1e30f;
    return ms;
  };
  std::map<int, float> tab_ms;                    // per table end layer
  std::map<std::pair<int, int>, float> mult_ms;  // per (table end layer, shape)
  float best_ms = 1e30f;
  for (int ml : kTabMinLogs) {
    const int te = tab_layers_end(k.log_d, k.log_lanes, k.start, ml);
    if (te > k.start && !twp) continue;
    if (!tab_ms.count(te))
      tab_ms[te] = te == k.start ? 0.f
                                 : time_of([&] { return run_tab_passes(d, twp, k.log_d, k.log_lanes, k.start, te, st); });
    for (int v = 0; v < kVariants; v++) {
      const auto key = std::make_pair(te, v);
      if (!mult_ms.count(key))
        mult_ms[key] = te == k.log_d ? 0.f : time_of([&] {
          return run_passes<true>(v, d, d, ~(size_t)0, tw, k.log_d, k.log_lanes, te, st);
        });
      const float t = tab_ms[te] + mult_ms[key];
      if (t < best_ms) {
        best_ms = t;
        best = TunedShape{te, v};
      }
    }
    // the deep-table pass, where the multiply part is exactly the last three layers
    if (twp && deep3_applies(k.log_d, k.log_lanes, te)) {
      const auto key = std::make_pair(te, kDeepVariant);
      if (!mult_ms.count(key)) mult_ms[key] = time_of([&] { return run_deep3(d, twp, tw, k.log_d, st); });
      const float t = tab_ms[te] + mult_ms[key];
      if (t < best_ms) {
        best_ms = t;
        best = TunedShape{te, kDeepVariant};
      }
    }
  }
  cudaStreamSynchronize(st);
  cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(scratch);
  return best;
}

TunedShape pick_shape(int log_d, int log_lanes, int start, const void* tw, const gf128* twp, cudaStream_t st) {
  const TunedShape dflt{tab_layers_end(log_d, log_lanes, start), kDefaultVariant};
  if (const char* f = std::getenv("FLOCK_NTT_VARIANT")) {  // a fixed shape, for measurements
    const int v = f[0] - '0';
    if ((v >= 0 && v < kVariants) || v == kDeepVariant) return TunedShape{dflt.tab_end, v};
  }
  if (!tuning_enabled()) return dflt;
  TuneKey k{0, log_d, log_lanes, start};
  cudaGetDevice(&k.dev);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(k);
    if (it != g_tuned.end()) return it->second;
  }
  const TunedShape sh = tune_shape(k, tw, twp, st);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[k] = sh;
  return sh;
}

}  // namespace

extern "C" int flock_ntt_tuned_variant(int device, int log_d, int log_lanes, int start_layer) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(TuneKey{device, log_d, log_lanes, start_layer});
  return it == g_tuned.end() ? -1 : it->second.variant;
}

extern "C" int flock_ntt_tuned_table_end(int device, int log_d, int log_lanes, int start_layer) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(TuneKey{device, log_d, log_lanes, start_layer});
  return it == g_tuned.end() ? -1 : it->second.tab_end;
}

extern "C" int flock_ntt_twiddle_classes(int log_d) {
  if (log_d < 1 || log_d > kMaxTwiddleClassLogD) return FLOCK_ERR_ARG;
  return flock_ntt_narrow_layers(log_d);
}

// Applies layers [start_layer, log_d) in passes whose shape the autotuner
// chose. d_src (may equal d_data) holds the input rows addressed with
// position mask 2^(log_d - start_layer) - 1, so a distinct d_src supplies the
// replicated message of a rate-1/2^start_layer code.
int flock_launch_ntt(void* d_data, const void* d_src, int log_d, int log_lanes, int start_layer,
                     cudaStream_t stream) {
  if (log_lanes < 3 || log_lanes > 10 || log_d < 1 || log_d > 30 || start_layer < 0 || start_layer > log_d)
    return FLOCK_ERR_SHAPE;
  const void* tw = flock_ntt_twiddles_prepared(log_d);
  if (!tw) return FLOCK_ERR_OOM;
  gf128* data = (gf128*)d_data;
  const gf128* src = d_src ? (const gf128*)d_src : data;
  size_t mask = d_src ? ((size_t)1 << (log_d - start_layer)) - 1 : ~(size_t)0;
  if (start_layer == log_d) {
    // No layers left: the output is the replicated source.
    if (src != data) {
      size_t row_bytes = ((size_t)1 << log_lanes) * 16;
      size_t chunk = (mask + 1) * row_bytes;
      for (size_t off = 0; off < ((size_t)1 << log_d) * row_bytes; off += chunk)
        if (cudaMemcpyAsync((char*)data + off, src, chunk, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
          return FLOCK_ERR_CUDA;
    }
    return FLOCK_OK;
  }
  // upper layers in table passes, then the multiply passes, of the tuned
  // depth and shape
  int l = start_layer;
  const gf128* twp = (const gf128*)flock_ntt_twiddles(log_d);
  if (!twp) return FLOCK_ERR_OOM;
  const TunedShape sh = pick_shape(log_d, log_lanes, start_layer, tw, twp, stream);
  const int tab_end = sh.tab_end;
  if (tab_end > l) {
    for (; l + 2 <= tab_end; l += 2) {
      int rc = launch_tab2(data, src, mask, twp, log_d, log_lanes, l, stream);
      if (rc != FLOCK_OK) return rc;
      src = data;
      mask = ~(size_t)0;
    }
  }
  if (l == log_d) return FLOCK_OK;
  if (sh.variant == kDeepVariant) {
    if (src == data && deep3_applies(log_d, log_lanes, l)) return run_deep3(data, twp, tw, log_d, stream);
    return run_passes<true>(kDefaultVariant, data, src, mask, tw, log_d, log_lanes, l, stream);
  }
  return run_passes<true>(sh.variant, data, src, mask, tw, log_d, log_lanes, l, stream);
}

// ---- NTT without device allocation -----------------------------------------
//
// Some callers cannot allocate device memory: a host framework that owns all
// of the GPU's memory through its own pool, or code running where cudaMalloc
// is not allowed (inside an allocator callback, or while a stream is being
// captured). flock_launch_ntt allocates a twiddle table per (device, log_d) on
// first use; flock_ntt_noalloc instead writes the table of each call into the
// fixed array below, which the module holds on every GPU that loads this
// library until the process exits.
//
// Every call shares the array and leaves its own table there. Each call
// rewrites all entries it reads before its passes read them, so nothing has to
// start at zero; but two calls whose work overlaps on the GPU (different
// streams, no ordering between them) overwrite each other's table and race.

namespace {

constexpr int kNoAllocMaxLogD = FLOCK_NTT_NOALLOC_MAX_LOG_D;

// Twiddle table of one transform of up to 2^16 positions: 2^16 - 1 entries
// of 16 bytes (1 MiB, the last entry unused).
__device__ __align__(256) gf128 g_noalloc_twiddles[(size_t)1 << kNoAllocMaxLogD];

// Device address of g_noalloc_twiddles per CUDA context, keyed by the
// context's process-unique id (cuCtxGetId): a context that a host framework
// destroys and creates again (cudaDeviceReset, a primary-context reset) gets a
// new id, and its first call looks the address up again.
std::mutex g_noalloc_mu;
std::map<unsigned long long, void*> g_noalloc_addr;

// Entry (layer, bit) of the breadth-first table's generators: for layer l the
// table holds the 2^l subset sums of {row_l[bit] : bit < l}, at
// v[l(l-1)/2 + bit]. 120 entries cover log_d = 16.
struct TwiddleGenerators {
  gf128 v[kNoAllocMaxLogD * (kNoAllocMaxLogD - 1) / 2];
};

__global__ void expand_twiddles_kernel(const __grid_constant__ TwiddleGenerators gen, int log_d,
                                       gf128* __restrict__ tw) {
  uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t total = (1u << log_d) - 1;
  if (idx >= total) return;
  int layer = 31 - __clz(idx + 1);
  uint32_t j = idx + 1 - (1u << layer);
  const gf128* row = gen.v + layer * (layer - 1) / 2;
  gf128 acc = gf_zero();
  for (int bit = 0; bit < layer; bit++)
    if ((j >> bit) & 1) acc = gf_add(acc, row[bit]);
  tw[idx] = acc;
}

// The same normalized subspace-polynomial rows as host_twiddles, in fixed
// arrays: gen row of layer l is ev[d - l - 1][1 .. l].
void twiddle_generators(int d, TwiddleGenerators* gen) {
  hf::F ev[kNoAllocMaxLogD][kNoAllocMaxLogD];
  for (int i = 0; i < d; i++) ev[0][i] = i < 64 ? hf::F(1ULL << i, 0) : hf::F(0, 1ULL << (i - 64));
  for (int i = 1; i < d; i++)
    for (int k = 1; k < d - i + 1; k++) ev[i][k - 1] = ev[i - 1][k] * (ev[i - 1][k] + ev[i - 1][0]);
  for (int i = 0; i < d; i++) {
    hf::F iv = hf::inv(ev[i][0]);
    for (int k = 0; k < d - i; k++) ev[i][k] = ev[i][k] * iv;
  }
  for (int layer = 1; layer < d; layer++) {
    const hf::F* row = ev[d - layer - 1];
    for (int bit = 0; bit < layer; bit++) {
      gf128& g = gen->v[layer * (layer - 1) / 2 + bit];
      g.w[0] = (uint32_t)row[bit + 1].lo;
      g.w[1] = (uint32_t)(row[bit + 1].lo >> 32);
      g.w[2] = (uint32_t)row[bit + 1].hi;
      g.w[3] = (uint32_t)(row[bit + 1].hi >> 32);
    }
  }
}

// Id of the current CUDA context (0 when none is current or the driver entry
// points are unavailable), through the runtime's driver entry points so the
// library links no driver library.
unsigned long long current_context_id() {
  typedef int (*GetCurrentFn)(CUcontext*);
  typedef int (*GetIdFn)(CUcontext, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetIdFn)f;
    cudaGetLastError();
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != 0 || !c || get_id(c, &id) != 0) return 0;
  return id;
}

// Device address of the scratch array in the current context: looked up with
// cudaGetSymbolAddress by the first call in each context (once per device
// unless its context is reset), read from the cache afterwards. A failed
// lookup clears the runtime's error state before it returns.
int noalloc_scratch(gf128** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  unsigned long long id = current_context_id();
  if (id) {
    auto it = g_noalloc_addr.find(id);
    if (it != g_noalloc_addr.end()) {
      *out = (gf128*)it->second;
      return FLOCK_OK;
    }
  }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_twiddles) != cudaSuccess || !p) {
    cudaGetLastError();
    return FLOCK_ERR_CUDA;
  }
  id = current_context_id();  // the lookup made the device's context current if none was
  if (id) g_noalloc_addr[id] = p;
  *out = (gf128*)p;
  return FLOCK_OK;
}

}  // namespace

extern "C" int flock_ntt_noalloc(void* d_data, int log_d, int log_num_ntts, int start_layer, void* stream) {
  if (!d_data) return FLOCK_ERR_ARG;
  if (log_d > kNoAllocMaxLogD) return FLOCK_ERR_LIMIT;
  if (log_num_ntts < 3 || log_num_ntts > 10 || log_d < 1 || start_layer < 0 || start_layer > log_d)
    return FLOCK_ERR_SHAPE;
  gf128* tw = nullptr;
  int rc = noalloc_scratch(&tw);
  if (rc != FLOCK_OK) return rc;
  if (start_layer == log_d) return FLOCK_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  TwiddleGenerators gen = {};
  twiddle_generators(log_d, &gen);
  uint32_t total = (1u << log_d) - 1;
  expand_twiddles_kernel<<<(total + 255) / 256, 256, 0, st>>>(gen, log_d, tw);
  flock_count_launch();
  if (cudaGetLastError() != cudaSuccess) return FLOCK_ERR_CUDA;
  gf128* data = (gf128*)d_data;
  int remaining = log_d - start_layer;
  int passes = (remaining + kMaxPassLayers - 1) / kMaxPassLayers;
  int l = start_layer;
  for (int q = 0; q < passes; q++) {
    int f = (remaining - (l - start_layer) + (passes - q) - 1) / (passes - q);
    rc = run_pass(f, data, data, ~(size_t)0, tw, log_d, log_num_ntts, l, st);
    if (rc != FLOCK_OK) return rc;
    l += f;
  }
  return FLOCK_OK;
}

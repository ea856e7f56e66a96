// BLAKE3 Merkle tree over equal-size leaves.
//
// Restates crates/flock-core/src/merkle.rs:200-235 and :706-817: a leaf is
// the non-root BLAKE3 chaining value of its bytes (one chunk: blocks with
// counter 0, CHUNK_START on the first and CHUNK_END on the last block, no
// ROOT; several chunks are merged into their BLAKE3 subtree without ROOT), a
// parent is the PARENT-flag compression of left||right under the IV. The tree
// is flat: leaves first, each level appended, root last.
//
// GB300 mapping: one thread per leaf with the chaining value in registers;
// each warp stages its 32 leaves' current 64-byte blocks through shared memory
// so the global reads are coalesced 2 KiB runs. Parent levels are reduced
// 512 nodes per CTA in shared memory (nine levels per launch).
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "blake3.cuh"
#include "flock_internal.h"

namespace {

constexpr int LEAF_THREADS = 128;
// Parent levels folded into the leaf kernel by shuffles (at most 5): a fused
// level runs one whole-warp compression for half as many parents as the level
// before, so five levels cost 160 lane-compressions for 31 parents of 32
// leaves, while the parent kernel (full warps over 512 nodes per CTA) does
// them in about 40 (the 2^20-leaf tree: 0.71 ms with five fused levels,
// 0.62 / 0.63 ms with one / two, 0.61 ms with none). The autotuner below
// picks among 0..kMaxTunedWarpLevels per tree shape; untuned calls use none.
constexpr int kMaxTunedWarpLevels = 2;

// Hashes `nblocks` 64-byte blocks of a chunk whose bytes this warp stages.
// data points at the first byte of this warp's 32 leaves' chunk; leaf_stride
// is the byte distance between consecutive leaves.
__device__ __forceinline__ void chunk_cv(const uint8_t* __restrict__ warp_base, size_t leaf_stride, int lane,
                                         int nlanes, uint32_t chunk_bytes, uint64_t chunk_counter, uint32_t* stage,
                                         uint32_t cv[8]) {
#pragma unroll
  for (int i = 0; i < 8; i++) cv[i] = b3::IV(i);
  uint32_t nblocks = (chunk_bytes + 63) / 64;
  for (uint32_t blk = 0; blk < nblocks; blk++) {
    uint32_t off = blk * 64;
    uint32_t len = chunk_bytes - off < 64 ? chunk_bytes - off : 64;
    // Stage block `blk` of all 32 leaves: 32 x 64 B, 16-byte granules.
    __syncwarp();
    if (len == 64 && nlanes == 32) {
      // whole blocks of a full warp: four unconditional 16-byte loads
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int q = lane + 32 * i, leaf = q >> 2, part = q & 3;
        reinterpret_cast<uint4*>(stage)[leaf * 4 + (leaf >> 1) + part] =
            *reinterpret_cast<const uint4*>(warp_base + (size_t)leaf * leaf_stride + off + part * 16);
      }
    } else
    for (int q = lane; q < 32 * 4; q += 32) {
      int leaf = q >> 2, part = q & 3;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (leaf < nlanes && (uint32_t)part * 16 < len) {
        const uint8_t* p = warp_base + (size_t)leaf * leaf_stride + off + part * 16;
        if (len - part * 16 >= 16) v = *reinterpret_cast<const uint4*>(p);
        else {
          uint32_t w[4] = {0, 0, 0, 0};
          for (uint32_t b = 0; b < len - part * 16; b++) w[b >> 2] |= (uint32_t)p[b] << (8 * (b & 3));
          v = make_uint4(w[0], w[1], w[2], w[3]);
        }
      }
      reinterpret_cast<uint4*>(stage)[leaf * 4 + (leaf >> 1) + part] = v;
    }
    __syncwarp();
    uint32_t m[16];
    const uint4* row = reinterpret_cast<const uint4*>(stage) + lane * 4 + (lane >> 1);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      uint4 v = row[q];
      m[4 * q] = v.x; m[4 * q + 1] = v.y; m[4 * q + 2] = v.z; m[4 * q + 3] = v.w;
    }
    uint32_t flags = (blk == 0 ? b3::CHUNK_START : 0u) | (blk + 1 == nblocks ? b3::CHUNK_END : 0u);
    uint32_t v16[16];
    b3::compress(cv, m, chunk_counter, len, flags, v16);
#pragma unroll
    for (int i = 0; i < 8; i++) cv[i] = v16[i];
  }
}

// Leaves, then `fuse` parent levels inside each warp (32 consecutive leaves:
// up to 5 levels) by shuffling the right child's chaining value to the left.
template <bool MULTI>
__global__ void __launch_bounds__(LEAF_THREADS)
leaf_kernel(const uint8_t* __restrict__ data, size_t n_leaves, uint32_t leaf_bytes, int fuse,
            uint32_t* __restrict__ out) {
  // 32 leaves x (4 + 0.5 padding) granules of 16 B per warp.
  __shared__ uint4 stage_all[(LEAF_THREADS / 32) * (32 * 4 + 16)];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t leaf0 = ((size_t)blockIdx.x * LEAF_THREADS) + warp * 32;
  if (leaf0 >= n_leaves) return;
  const int nlanes = n_leaves - leaf0 >= 32 ? 32 : (int)(n_leaves - leaf0);
  uint32_t* stage = reinterpret_cast<uint32_t*>(stage_all + warp * (32 * 4 + 16));
  const uint8_t* base = data + leaf0 * leaf_bytes;
  uint32_t cv[8];
  if (!MULTI) {
    chunk_cv(base, leaf_bytes, lane, nlanes, leaf_bytes, 0, stage, cv);
  } else {
    // Whole chunks; merge with the BLAKE3 chaining-value stack.
    uint32_t nchunks = leaf_bytes / 1024;
    uint32_t stack[4][8];
    int depth = 0;
    for (uint32_t c = 0; c < nchunks; c++) {
      uint32_t ccv[8];
      chunk_cv(base + (size_t)c * 1024, leaf_bytes, lane, nlanes, 1024, c, stage, ccv);
      if (c + 1 < nchunks) {
        uint64_t total = c + 1;
        while ((total & 1) == 0) {
          uint32_t m[16];
#pragma unroll
          for (int i = 0; i < 8; i++) { m[i] = stack[depth - 1][i]; m[8 + i] = ccv[i]; }
#pragma unroll
          for (int i = 0; i < 8; i++) ccv[i] = b3::IV(i);
          b3::compress_cv(ccv, m, 64, b3::PARENT);
          depth--;
          total >>= 1;
        }
#pragma unroll
        for (int i = 0; i < 8; i++) stack[depth][i] = ccv[i];
        depth++;
      } else {
        for (int d = depth - 1; d >= 0; d--) {
          uint32_t m[16];
#pragma unroll
          for (int i = 0; i < 8; i++) { m[i] = stack[d][i]; m[8 + i] = ccv[i]; }
#pragma unroll
          for (int i = 0; i < 8; i++) ccv[i] = b3::IV(i);
          b3::compress_cv(ccv, m, 64, b3::PARENT);
        }
      }
      if (c + 1 == nchunks) {
#pragma unroll
        for (int i = 0; i < 8; i++) cv[i] = ccv[i];
      }
    }
  }
  if (lane < nlanes) {
    uint4* o = reinterpret_cast<uint4*>(out + (leaf0 + lane) * 8);
    o[0] = make_uint4(cv[0], cv[1], cv[2], cv[3]);
    o[1] = make_uint4(cv[4], cv[5], cv[6], cv[7]);
  }
  // fused parent levels (only when the warp holds 32 whole leaves)
  size_t lvl_off = 0, lvl_len = n_leaves, idx = leaf0 + lane;
  for (int l = 1; l <= fuse; l++) {
    const int step = 1 << (l - 1);
    uint32_t rc[8];
#pragma unroll
    for (int i = 0; i < 8; i++) rc[i] = __shfl_down_sync(0xffffffffu, cv[i], step);
    bool left = (lane & (2 * step - 1)) == 0;
    if (left) {
      uint32_t m[16];
#pragma unroll
      for (int i = 0; i < 8; i++) { m[i] = cv[i]; m[8 + i] = rc[i]; }
#pragma unroll
      for (int i = 0; i < 8; i++) cv[i] = b3::IV(i);
      b3::compress_cv(cv, m, 64, b3::PARENT);
    }
    lvl_off += lvl_len;
    lvl_len >>= 1;
    idx >>= 1;
    if (left) {
      uint4* o = reinterpret_cast<uint4*>(out + (lvl_off + idx) * 8);
      o[0] = make_uint4(cv[0], cv[1], cv[2], cv[3]);
      o[1] = make_uint4(cv[4], cv[5], cv[6], cv[7]);
    }
  }
}

// Reduces 2*blockDim consecutive nodes of one level into up to `levels`
// parent levels. in: level start; outs: start of the next level; the level
// after that follows contiguously in the flat layout.
constexpr int PARENT_THREADS = 256;
__global__ void __launch_bounds__(PARENT_THREADS)
parent_kernel(uint32_t* __restrict__ tree, size_t level_off, size_t level_len, int levels) {
  __shared__ uint32_t nodes[2 * PARENT_THREADS * 8 + 2 * PARENT_THREADS];
  const int t = threadIdx.x;
  const size_t base = (size_t)blockIdx.x * 2 * PARENT_THREADS;
  size_t span = level_len - base < (size_t)(2 * PARENT_THREADS) ? level_len - base : (size_t)(2 * PARENT_THREADS);
  // load span nodes (padded rows of 9 words to avoid conflicts)
  for (size_t e = t; e < span * 8; e += PARENT_THREADS) {
    size_t node = e >> 3;
    nodes[node * 9 + (e & 7)] = tree[(level_off + base + node) * 8 + (e & 7)];
  }
  __syncthreads();
  size_t in_off = level_off, in_len = level_len, cur = span;
  size_t blk_base = base;
  for (int l = 0; l < levels && cur > 1; l++) {
    size_t out_off = in_off + in_len;
    size_t out_len = in_len >> 1;
    size_t n_out = cur >> 1;
    uint32_t cv[8];
    bool act = (size_t)t < n_out;
    if (act) {
      uint32_t m[16];
#pragma unroll
      for (int i = 0; i < 8; i++) { m[i] = nodes[(2 * t) * 9 + i]; m[8 + i] = nodes[(2 * t + 1) * 9 + i]; }
#pragma unroll
      for (int i = 0; i < 8; i++) cv[i] = b3::IV(i);
      b3::compress_cv(cv, m, 64, b3::PARENT);
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int i = 0; i < 8; i++) nodes[t * 9 + i] = cv[i];
      size_t gi = out_off + (blk_base >> 1) + t;
      uint4* o = reinterpret_cast<uint4*>(tree + gi * 8);
      o[0] = make_uint4(cv[0], cv[1], cv[2], cv[3]);
      o[1] = make_uint4(cv[4], cv[5], cv[6], cv[7]);
    }
    __syncthreads();
    in_off = out_off;
    in_len = out_len;
    cur = n_out;
    blk_base >>= 1;
  }
}

}  // namespace

namespace {

// The leaf kernel with `levels` fused parent levels (fewer where the tree or
// a warp's 32 leaves have fewer), then the parent kernels up to the root.
int launch_tree(const void* d_data, size_t n_leaves, size_t leaf_bytes, void* d_tree, int levels, cudaStream_t st) {
  size_t blocks = (n_leaves + LEAF_THREADS - 1) / LEAF_THREADS;
  int fuse = 0;
  while (fuse < levels && ((size_t)2 << fuse) <= n_leaves) fuse++;  // levels inside a warp of 32 leaves
  if (n_leaves < 32) fuse = 0;
  if (leaf_bytes <= 1024)
    leaf_kernel<false><<<(unsigned)blocks, LEAF_THREADS, 0, st>>>((const uint8_t*)d_data, n_leaves,
                                                                  (uint32_t)leaf_bytes, fuse, (uint32_t*)d_tree);
  else
    leaf_kernel<true><<<(unsigned)blocks, LEAF_THREADS, 0, st>>>((const uint8_t*)d_data, n_leaves,
                                                                 (uint32_t)leaf_bytes, fuse, (uint32_t*)d_tree);
  flock_count_launch();
  if (cudaGetLastError() != cudaSuccess) return FLOCK_ERR_CUDA;
  size_t off = 0, len = n_leaves;
  for (int i = 0; i < fuse; i++) {
    off += len;
    len >>= 1;
  }
  while (len > 1) {
    int lv = 0;
    size_t per = 2 * PARENT_THREADS;
    size_t span = len < per ? len : per;
    while (((size_t)1 << (lv + 1)) <= span) lv++;  // log2(span)
    size_t grid = (len + per - 1) / per;
    parent_kernel<<<(unsigned)grid, PARENT_THREADS, 0, st>>>((uint32_t*)d_tree, off, len, lv); flock_count_launch();
    if (cudaGetLastError() != cudaSuccess) return FLOCK_ERR_CUDA;
    for (int i = 0; i < lv; i++) {
      off += len;
      len >>= 1;
    }
  }
  return FLOCK_OK;
}

// ---- autotuner: fused parent levels per tree shape --------------------------
//
// The first tree of a (device, leaves, leaf bytes) shape with at least
// kTuneMinLeaves leaves is built once per candidate level count (every build
// writes the same tree, so the caller's tree is final whichever is last), timed
// with CUDA events on the caller's stream; later trees of the shape use the
// fastest. FLOCK_MERKLE_TUNE=0 in the environment turns tuning off.
constexpr size_t kTuneMinLeaves = (size_t)1 << 12;
struct MerkleKey {
  int dev;
  size_t leaves, leaf_bytes;
  bool operator<(const MerkleKey& o) const {
    return std::tie(dev, leaves, leaf_bytes) < std::tie(o.dev, o.leaves, o.leaf_bytes);
  }
};
std::mutex g_mtune_mu;
std::map<MerkleKey, int> g_mtuned;

bool merkle_tuning_enabled() {
  const char* e = std::getenv("FLOCK_MERKLE_TUNE");
  return !(e && e[0] == '0');
}

}  // namespace

extern "C" int flock_merkle_tuned_levels(int device, size_t n_leaves, size_t leaf_bytes) {
  std::lock_guard<std::mutex> lk(g_mtune_mu);
  auto it = g_mtuned.find(MerkleKey{device, n_leaves, leaf_bytes});
  return it == g_mtuned.end() ? -1 : it->second;
}

int flock_launch_merkle(const void* d_data, size_t n_leaves, size_t leaf_bytes, void* d_tree, cudaStream_t st) {
  if (n_leaves == 0 || (n_leaves & (n_leaves - 1)) || leaf_bytes == 0 || leaf_bytes % 16 ||
      (leaf_bytes > 1024 && (leaf_bytes % 1024 || leaf_bytes > 4096)))
    return FLOCK_ERR_SHAPE;
  if (n_leaves < kTuneMinLeaves || !merkle_tuning_enabled()) return launch_tree(d_data, n_leaves, leaf_bytes, d_tree, 0, st);
  MerkleKey k{0, n_leaves, leaf_bytes};
  cudaGetDevice(&k.dev);
  {
    std::lock_guard<std::mutex> lk(g_mtune_mu);
    auto it = g_mtuned.find(k);
    if (it != g_mtuned.end()) return launch_tree(d_data, n_leaves, leaf_bytes, d_tree, it->second, st);
  }
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return FLOCK_ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return FLOCK_ERR_CUDA;
  }
  int best = 0, rc = FLOCK_OK;
  float best_ms = 1e30f;
  for (int levels = 0; levels <= kMaxTunedWarpLevels && rc == FLOCK_OK; levels++) {
    cudaEventRecord(e0, st);
    rc = launch_tree(d_data, n_leaves, leaf_bytes, d_tree, levels, st);
    cudaEventRecord(e1, st);
    float ms = 0;
    if (rc == FLOCK_OK && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
        ms < best_ms) {
      best_ms = ms;
      best = levels;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != FLOCK_OK) return rc;
  std::lock_guard<std::mutex> lk(g_mtune_mu);
  g_mtuned[k] = best;
  return FLOCK_OK;
}

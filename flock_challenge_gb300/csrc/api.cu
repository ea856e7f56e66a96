// C ABI entry points (include/flock_gpu.h) over the CUDA kernels.
#include <cstring>
#include <new>
#include <vector>

#include "flock_internal.h"
#include "prover.h"
#include "r1cs_setup.h"

#include <atomic>
#include <mutex>
#include <set>

static std::atomic<unsigned long long> g_launches{0};
void flock_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void flock_once_per_device(const void* key, void (*fn)()) {
  static std::mutex mu;
  static std::set<std::pair<int, const void*>> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  // run under the lock: no thread launches the kernel before the work is done
  if (done.insert({dev, key}).second) fn();
}

struct flock_ctx {
  int device = 0;
  size_t hbm_budget = 0;
  ProverState* prover = nullptr;
  std::vector<uint8_t> last_proof;
};

namespace {
inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
}  // namespace

extern "C" {

const char* flock_version(void) { return "flock-gb300 0.1 (sm_103a)"; }

uint64_t flock_kernel_launches(void) { return g_launches.load(); }

int flock_create(int device, size_t hbm_budget, flock_ctx** out) {
  if (!out) return FLOCK_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return FLOCK_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return FLOCK_ERR_CUDA;
  flock_ctx* c = new (std::nothrow) flock_ctx;
  if (!c) return FLOCK_ERR_OOM;
  c->device = device;
  c->hbm_budget = hbm_budget;
  *out = c;
  return FLOCK_OK;
}

void flock_destroy(flock_ctx* ctx) {
  if (!ctx) return;
  flock_prover_destroy(ctx->prover);
  delete ctx;
}

int flock_witness(const flock_compression* d_in, size_t n, int n_blocks_log, void* d_z, void* d_a, void* d_b,
                  void* d_stripe, void* stream) {
  if (!d_z || (n > 0 && !d_in) || n_blocks_log < 3 || n_blocks_log > 24) return FLOCK_ERR_ARG;
  return flock_launch_witness(d_in, n, n_blocks_log, d_z, d_a, d_b, d_stripe, as_stream(stream));
}

int flock_ntt(flock_ctx* ctx, void* d_data, int log_d, int log_num_ntts, int start_layer, void* stream) {
  if (!ctx || !d_data) return FLOCK_ERR_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return FLOCK_ERR_CUDA;
  return flock_launch_ntt(d_data, nullptr, log_d, log_num_ntts, start_layer, as_stream(stream));
}

int flock_merkle_tree(const void* d_data, size_t n_leaves, size_t leaf_bytes, void* d_tree, void* stream) {
  if (!d_data || !d_tree) return FLOCK_ERR_ARG;
  return flock_launch_merkle(d_data, n_leaves, leaf_bytes, d_tree, as_stream(stream));
}

int flock_commit(flock_ctx* ctx, const void* d_z, int m, int log_inv_rate, int log_batch_size, void* d_codeword,
                 void* d_tree, uint8_t root[32], void* stream) {
  if (!ctx || !d_z || !d_codeword || !d_tree) return FLOCK_ERR_ARG;
  if (m < 7 + log_batch_size + 1 || log_inv_rate < 1 || log_batch_size < 4 || log_batch_size > 10)
    return FLOCK_ERR_SHAPE;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return FLOCK_ERR_CUDA;
  cudaStream_t st = as_stream(stream);
  int log_d = m - 7 - log_batch_size + log_inv_rate;
  int rc = flock_launch_ntt(d_codeword, d_z, log_d, log_batch_size, log_inv_rate, st);
  if (rc != FLOCK_OK) return rc;
  size_t n_leaves = (size_t)1 << log_d;
  rc = flock_launch_merkle(d_codeword, n_leaves, (size_t)16 << log_batch_size, d_tree, st);
  if (rc != FLOCK_OK) return rc;
  if (root) {
    const uint8_t* d_root = (const uint8_t*)d_tree + (2 * n_leaves - 2) * 32;
    if (cudaMemcpyAsync(root, d_root, 32, cudaMemcpyDeviceToHost, st) != cudaSuccess) return FLOCK_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return FLOCK_ERR_CUDA;
  }
  return FLOCK_OK;
}

int flock_setup(flock_ctx* ctx, size_t n_blocks) {
  if (!ctx || n_blocks == 0 || n_blocks > ((size_t)1 << 24)) return FLOCK_ERR_ARG;
  size_t n = n_blocks < 8 ? 8 : n_blocks;
  int n_log = 0;
  while (((size_t)1 << n_log) < n) n_log++;
  uint8_t d[32];
  flock_statement_digest(14 + n_log, d);
  flock_host_csc();
  if (!ctx->prover) ctx->prover = flock_prover_create(ctx->device);
  return ctx->prover ? FLOCK_OK : FLOCK_ERR_CUDA;
}

static int prove_impl(flock_ctx* ctx, const flock_compression* in, size_t n, uint8_t* out, size_t cap, size_t* len,
                      bool on_device) {
  if (!ctx || !len || (n && !in)) return FLOCK_ERR_ARG;
  size_t nn = n < 8 ? 8 : n;
  int n_log = 0;
  while (((size_t)1 << n_log) < nn) n_log++;
  if (ctx->hbm_budget && flock_footprint_bytes((uint32_t)n_log) > ctx->hbm_budget) return FLOCK_ERR_OOM;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  int rc = flock_prover_prove(ctx->prover, in, n, n_log, ctx->last_proof, on_device);
  if (rc != FLOCK_OK) return rc;
  *len = ctx->last_proof.size();
  if (!out || cap < ctx->last_proof.size()) return FLOCK_ERR_CAPACITY;
  memcpy(out, ctx->last_proof.data(), ctx->last_proof.size());
  return FLOCK_OK;
}

int flock_prove(flock_ctx* ctx, const flock_compression* in, size_t n, uint8_t* out, size_t cap, size_t* len) {
  return prove_impl(ctx, in, n, out, cap, len, false);
}

int flock_prove_device(flock_ctx* ctx, const flock_compression* d_in, size_t n, uint8_t* out, size_t cap,
                       size_t* len) {
  return prove_impl(ctx, d_in, n, out, cap, len, true);
}

int flock_generate_inputs(uint32_t log2_size, uint64_t seed, void* d_out, void* stream) {
  if (!d_out || log2_size > 30) return FLOCK_ERR_ARG;
  uint64_t l = log2_size;
  return flock_launch_gen_inputs(seed ^ ((l << 29) | (l >> 35)), (size_t)1 << log2_size, d_out, as_stream(stream));
}

int flock_prove_seed(flock_ctx* ctx, uint32_t log2_size, uint64_t seed, uint8_t* out, size_t cap, size_t* len) {
  if (!ctx || !len || log2_size < 8 || log2_size > 21) return FLOCK_ERR_ARG;
  if (ctx->hbm_budget && flock_footprint_bytes(log2_size) > ctx->hbm_budget) return FLOCK_ERR_OOM;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  int rc = flock_prover_prove_seed(ctx->prover, (int)log2_size, seed, ctx->last_proof);
  if (rc != FLOCK_OK) return rc;
  *len = ctx->last_proof.size();
  if (!out || cap < ctx->last_proof.size()) return FLOCK_ERR_CAPACITY;
  memcpy(out, ctx->last_proof.data(), ctx->last_proof.size());
  return FLOCK_OK;
}

int flock_verify(flock_ctx* ctx, const uint8_t* proof, size_t len, int* accepted) {
  if (!ctx || (!proof && len) || !accepted) return FLOCK_ERR_ARG;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  return flock_prover_verify(ctx->prover, proof, len, accepted, nullptr);
}

int flock_verify_batch(flock_ctx* ctx, size_t count, const uint8_t* const* proofs, const size_t* lens, int* accepted) {
  if (!ctx || (count && (!proofs || !lens || !accepted))) return FLOCK_ERR_ARG;
  for (size_t i = 0; i < count; i++) {
    int rc = flock_verify(ctx, proofs[i], lens[i], &accepted[i]);
    if (rc != FLOCK_OK) return rc;
  }
  return FLOCK_OK;
}

void* flock_stream(flock_ctx* ctx) {
  if (!ctx) return nullptr;
  if (!ctx->prover) ctx->prover = flock_prover_create(ctx->device);
  return ctx->prover ? (void*)flock_prover_stream(ctx->prover) : nullptr;
}

int flock_last_phase_times(const flock_ctx* ctx, double* ms, int n) {
  if (!ctx || !ctx->prover || !ms) return FLOCK_ERR_ARG;
  const FlockPhaseTimes& t = flock_prover_times(ctx->prover);
  double v[8] = {t.setup_ms, t.commit_ms, t.zc_round1_ms, t.zc_rounds_ms, t.lincheck_ms, t.ring_switch_ms,
                 t.ligerito_ms, t.serialize_ms};
  for (int i = 0; i < n && i < 8; i++) ms[i] = v[i];
  return FLOCK_OK;
}

}  // extern "C"

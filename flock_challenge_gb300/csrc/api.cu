// C ABI entry points (include/flock_gpu.h) over the CUDA kernels.
#include <cstring>
#include <new>

#include "flock_internal.h"

struct flock_ctx {
  int device = 0;
  size_t hbm_budget = 0;
};

namespace {
inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
}  // namespace

extern "C" {

const char* flock_version(void) { return "flock-gb300 0.1 (sm_103a)"; }

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

void flock_destroy(flock_ctx* ctx) { delete ctx; }

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

}  // extern "C"

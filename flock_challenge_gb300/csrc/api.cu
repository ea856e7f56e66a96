// C ABI entry points (include/flock_gpu.h) over the CUDA kernels.
#include <cstring>
#include <new>
#include <vector>

#include "flock_internal.h"
#include "prover.h"
#include "host_blake3.h"
#include "r1cs_setup.h"
#include "transcript.h"

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

struct flock_transcript {
  fs::Transcript t;
};

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

int flock_transcript_create(const uint8_t* domain, size_t domain_len, flock_transcript** out) {
  if (!out || (!domain && domain_len)) return FLOCK_ERR_ARG;
  *out = new (std::nothrow) flock_transcript{fs::Transcript(std::string((const char*)domain, domain_len))};
  return *out ? FLOCK_OK : FLOCK_ERR_OOM;
}

int flock_transcript_fork(const flock_transcript* t, flock_transcript** out) {
  if (!t || !out) return FLOCK_ERR_ARG;
  *out = new (std::nothrow) flock_transcript{t->t};
  return *out ? FLOCK_OK : FLOCK_ERR_OOM;
}

void flock_transcript_destroy(flock_transcript* t) { delete t; }

int flock_transcript_observe_label(flock_transcript* t, const uint8_t* label, size_t len) {
  if (!t || (!label && len)) return FLOCK_ERR_ARG;
  t->t.label(label, len);
  return FLOCK_OK;
}

int flock_transcript_observe_f128(flock_transcript* t, const uint64_t value[2]) {
  if (!t || !value) return FLOCK_ERR_ARG;
  t->t.observe(hf::F(value[0], value[1]));
  return FLOCK_OK;
}

int flock_transcript_observe_f128_slice(flock_transcript* t, const uint64_t* values, size_t n) {
  if (!t || (!values && n)) return FLOCK_ERR_ARG;
  std::vector<hf::F> v(n);
  for (size_t i = 0; i < n; i++) v[i] = hf::F(values[2 * i], values[2 * i + 1]);
  t->t.observe_slice(v.data(), n);
  return FLOCK_OK;
}

int flock_transcript_observe_bytes(flock_transcript* t, const uint8_t* bytes, size_t len) {
  if (!t || (!bytes && len)) return FLOCK_ERR_ARG;
  t->t.observe_bytes(bytes, len);
  return FLOCK_OK;
}

int flock_transcript_sample_f128(flock_transcript* t, uint64_t out[2]) {
  if (!t || !out) return FLOCK_ERR_ARG;
  hf::F v = t->t.sample();
  out[0] = v.lo;
  out[1] = v.hi;
  return FLOCK_OK;
}

int flock_transcript_sample_f128_vec(flock_transcript* t, size_t n, uint64_t* out) {
  if (!t || (!out && n)) return FLOCK_ERR_ARG;
  auto v = t->t.sample_vec(n);
  for (size_t i = 0; i < n; i++) {
    out[2 * i] = v[i].lo;
    out[2 * i + 1] = v[i].hi;
  }
  return FLOCK_OK;
}

int flock_prove_challenger(flock_ctx* ctx, const flock_compression* in, size_t n, int in_on_device,
                           flock_transcript* tr, uint8_t* out, size_t cap, size_t* len, uint8_t root[32],
                           flock_r1cs_claim* claim) {
  if (!ctx || !len || !tr || (n && !in)) return FLOCK_ERR_ARG;
  size_t nn = n < 8 ? 8 : n;
  int n_log = 0;
  while (((size_t)1 << n_log) < nn) n_log++;
  if (ctx->hbm_budget && flock_footprint_bytes((uint32_t)n_log) > ctx->hbm_budget) return FLOCK_ERR_OOM;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  // the proof runs on a copy, so a too-small output buffer leaves `tr` as it was
  fs::Transcript work = tr->t;
  flock_r1cs_claim cl;
  int rc = flock_prover_prove(ctx->prover, in, n, n_log, ctx->last_proof, in_on_device != 0, nullptr, &work, &cl);
  if (rc != FLOCK_OK) return rc;
  *len = ctx->last_proof.size();
  if (!out || cap < ctx->last_proof.size()) return FLOCK_ERR_CAPACITY;
  memcpy(out, ctx->last_proof.data(), ctx->last_proof.size());
  if (root) memcpy(root, ctx->last_proof.data() + 7, 32);  // "FLOCK" 4 2, then Commitment.root
  if (claim) *claim = cl;
  tr->t = work;
  return FLOCK_OK;
}

int flock_verify_challenger(flock_ctx* ctx, const uint8_t* proof, size_t len, flock_transcript* tr, int* accepted) {
  if (!ctx || !tr || (!proof && len) || !accepted) return FLOCK_ERR_ARG;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  return flock_prover_verify(ctx->prover, proof, len, accepted, nullptr, &tr->t);
}

int flock_prove_chain(flock_ctx* ctx, const flock_compression* in, size_t n, const char* domain, uint8_t* out,
                      size_t cap, size_t* len) {
  if (!ctx || !len || !in) return FLOCK_ERR_ARG;
  if (n < 256 || n > ((size_t)1 << 21) || (n & (n - 1))) return FLOCK_ERR_SHAPE;
  int n_log = 0;
  while (((size_t)1 << n_log) < n) n_log++;
  if (ctx->hbm_budget && flock_footprint_bytes((uint32_t)n_log) > ctx->hbm_budget) return FLOCK_ERR_OOM;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  ChainReq req;
  if (domain) req.domain = domain;
  memcpy(req.cv0, in[0].cv, 32);
  uint32_t o[16];
  const flock_compression& l = in[n - 1];
  hb3::compress(l.cv, l.m, l.counter, l.block_len, l.flags, o);
  memcpy(req.cv_last, o, 32);
  int rc = flock_prover_prove(ctx->prover, in, n, n_log, ctx->last_proof, false, &req);
  if (rc != FLOCK_OK) return rc;
  *len = ctx->last_proof.size();
  if (!out || cap < ctx->last_proof.size()) return FLOCK_ERR_CAPACITY;
  memcpy(out, ctx->last_proof.data(), ctx->last_proof.size());
  return FLOCK_OK;
}

int flock_verify_chain(flock_ctx* ctx, const uint8_t* bundle, size_t len, const char* domain, int* accepted) {
  if (!ctx || (!bundle && len) || !accepted) return FLOCK_ERR_ARG;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  return flock_prover_verify_chain(ctx->prover, bundle, len, domain, accepted, nullptr);
}

int flock_chain_inputs(size_t steps, uint64_t seed, const uint32_t* cv0, flock_compression* out) {
  if (!out && steps) return FLOCK_ERR_ARG;
  static const uint32_t kIV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                                  0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
  uint32_t cv[8];
  memcpy(cv, cv0 ? cv0 : kIV, 32);
  uint64_t s = seed;
  for (size_t i = 0; i < steps; i++) {
    flock_compression& c = out[i];
    memcpy(c.cv, cv, 32);
    for (int j = 0; j < 16; j++) {
      s += 0x9E3779B97F4A7C15ull;
      uint64_t z = s;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      c.m[j] = (uint32_t)(z ^ (z >> 31));
    }
    c.counter = 0;
    c.block_len = 64;
    c.flags = 0;
    uint32_t o[16];
    hb3::compress(c.cv, c.m, 0, 64, 0, o);
    memcpy(cv, o, 32);
  }
  return FLOCK_OK;
}

void* flock_stream(flock_ctx* ctx) {
  if (!ctx) return nullptr;
  if (!ctx->prover) ctx->prover = flock_prover_create(ctx->device);
  return ctx->prover ? (void*)flock_prover_stream(ctx->prover) : nullptr;
}

int flock_kernel_timing(flock_ctx* ctx, int enable) {
  if (!ctx) return FLOCK_ERR_ARG;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  return flock_prover_set_timing(ctx->prover, enable != 0);
}

int flock_set_wait_limit(flock_ctx* ctx, double limit_ms) {
  if (!ctx) return FLOCK_ERR_ARG;
  if (!ctx->prover) {
    ctx->prover = flock_prover_create(ctx->device);
    if (!ctx->prover) return FLOCK_ERR_CUDA;
  }
  return flock_prover_set_wait_limit(ctx->prover, limit_ms);
}

int flock_last_kernel_times(const flock_ctx* ctx, double* ms, int n) {
  if (!ctx || !ctx->prover || !ms) return FLOCK_ERR_ARG;
  return flock_prover_kernel_times(ctx->prover, ms, n);
}

int flock_last_phase_times(const flock_ctx* ctx, double* ms, int n) {
  if (!ctx || !ctx->prover || !ms) return FLOCK_ERR_ARG;
  const FlockPhaseTimes& t = flock_prover_times(ctx->prover);
  double v[8] = {t.setup_ms, t.commit_ms, t.zc_round1_ms, t.zc_rounds_ms, t.lincheck_ms, t.ring_switch_ms,
                 t.ligerito_ms, t.serialize_ms};
  for (int i = 0; i < n && i < 8; i++) ms[i] = v[i];
  return FLOCK_OK;
}

int flock_last_host_waits(const flock_ctx* ctx, uint64_t* waits, double* blocked_ms, int n) {
  if (!ctx || !ctx->prover || !waits || !blocked_ms) return FLOCK_ERR_ARG;
  const FlockPhaseTimes& t = flock_prover_times(ctx->prover);
  for (int i = 0; i < n && i < 8; i++) {
    waits[i] = t.waits[i];
    blocked_ms[i] = t.blocked_ms[i];
  }
  return FLOCK_OK;
}

}  // extern "C"

// Internal declarations shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/flock_gpu.h"
#include "stream_wait.h"

constexpr int FLOCK_K_LOG = 14;
constexpr int FLOCK_K = 1 << FLOCK_K_LOG;

int flock_launch_witness(const flock_compression* d_in, size_t n_in, int n_blocks_log, void* d_z, void* d_a,
                         void* d_b, void* d_stripe, cudaStream_t stream);

// NTT twiddle tables: device copy of the breadth-first table for a domain of
// 2^log_d (layer l at offset 2^l - 1), built on the host once per size.
const void* flock_ntt_twiddles(int log_d);
int flock_launch_ntt(void* d_data, const void* d_src, int log_d, int log_num_ntts, int start_layer,
                     cudaStream_t stream);

int flock_launch_merkle(const void* d_data, size_t n_leaves, size_t leaf_bytes, void* d_tree,
                        cudaStream_t stream);

// ---- protocol kernels ------------------------------------------------------
struct ZcRound1Tables;
// eq_basis: n_outer x 8 F128 from flock_launch_zc1_eq_basis.
int flock_launch_zc_round1(const void* a, const void* b, const void* c, size_t n_outer, const void* eq_basis,
                           const ZcRound1Tables* d_tables, void* partials, int grid, cudaStream_t st);
// out[8 xo + k] = phi8(2^k) eq_out[xo] for xo < n_outer (round 1's table basis).
int flock_launch_zc1_eq_basis(const void* eq_out, size_t n_outer, const ZcRound1Tables* d_tables, void* out,
                              cudaStream_t st);
int flock_launch_reduce_rows(const void* in, size_t count, int width, void* out, cudaStream_t st);
int flock_launch_eq_split(const void* r, int lo_bits, int hi_bits, void* lo, void* hi, cudaStream_t st);
// Several eq table pairs in one launch (device array of jobs; lo_bits and
// hi_bits each at most 28; max_entries = the largest 2^lo_bits + 2^hi_bits).
struct FlockEqJob {
  const void* r;
  void* lo;
  void* hi;
  int lo_bits, hi_bits;
};
int flock_launch_eq_split_multi(const FlockEqJob* d_jobs, int n_jobs, size_t max_entries, cudaStream_t st);
int flock_launch_zc_round(const void* A, const void* B, size_t n_pairs, int bind, const uint64_t rho[2], void* Aout,
                          void* Bout, const void* eq_lo, const void* eq_hi, int lo_bits, void* partials, int grid,
                          cudaStream_t st);
int flock_launch_bind_pairs(const void* A, const void* B, size_t n, const uint64_t rho[2], void* Aout, void* Bout,
                            cudaStream_t st);

int flock_launch_lc_partial_fold(const void* stripe, size_t n_stripes, const void* eq_lo, const void* eq_hi,
                                 int lo_bits, void* partials, int grid, cudaStream_t st);
int flock_launch_lc_comb(const uint32_t* a_ptr, const uint32_t* a_idx, const uint32_t* b_ptr,
                         const uint32_t* b_idx, const void* eq, const uint64_t alpha[2], const uint64_t beta[2],
                         int pin, void* comb, cudaStream_t st);
int flock_launch_lc_quirky_eq(const void* lag, const void* x_rest, int n_rest, void* out, cudaStream_t st);

// scratch: 32 x 128 F128 of partial sums
int flock_launch_shv_from_zvec(const void* zvec, const void* eq_tail, void* scratch, void* out, cudaStream_t st);
// The combined basis fused with the first Ligerito message over (f, b):
// partials (u0, u2, 0) per block, flock_combined_basis_msg_grid(n, lo_bits) blocks.
int flock_combined_basis_msg_grid(size_t n, int lo_bits);
int flock_launch_combined_basis_msg(size_t n, const void* t0_lo, const void* t0_hi, const void* t1_lo,
                                    const void* t1_hi, int lo_bits, const void* w, const void* f, void* b,
                                    void* partials, cudaStream_t st);
int flock_launch_combined_basis(size_t n, const void* t0_lo, const void* t0_hi, const void* t1_lo,
                                const void* t1_hi, int lo_bits, const void* tables, void* b, cudaStream_t st);

int flock_lig_grid(size_t n_pairs);
int flock_launch_lig_fold_msg(const void* f, const void* b, size_t n_out, int fold, const uint64_t r[2], void* fo,
                              void* bo, void* partials, int grid, cudaStream_t st);
int flock_launch_lig_intro_eq(const void* f, size_t n, const void* lo, const void* hi, int lo_bits, void* partials,
                              int grid, cudaStream_t st);
int flock_launch_glue_eq(void* b, size_t n, const void* lo, const void* hi, int lo_bits, const uint64_t beta[2],
                         cudaStream_t st);
int flock_launch_glue(void* b, const void* add, size_t n, const uint64_t beta[2], cudaStream_t st);
// LO holds nq << flock_induce_basis_lo_bits(n) entries, HI nq << (n - that).
int flock_induce_basis_lo_bits(int n);
// what_lin: [n][32] F128, What_k(x^b) (the normalized subspace polynomials on
// the index bits; What_k(q) is their XOR over the set bits of q).
// scratch: flock_induce_basis_scratch_bytes(n) bytes (slice partials of small bases)
size_t flock_induce_basis_scratch_bytes(int n);
int flock_launch_induce_basis(const uint32_t* d_queries, int nq, int n, const void* what_lin, const void* alpha_w,
                              void* W, void* LO, void* HI, void* basis, void* scratch, cudaStream_t st);
int flock_launch_gather_rows(const void* mat, const uint32_t* rows, int n_rows, int width, void* out,
                             cudaStream_t st);
int flock_launch_gather_nodes(const void* tree, const uint32_t* idx, int n, void* out, cudaStream_t st);
// waits: the caller's count of host waits (nullptr: not counted).
int flock_grind(const uint8_t digest[32], uint32_t bits, void* d_scratch, int* parity, uint64_t* h_best,
                cudaStream_t st, WaitStats* waits, uint64_t* nonce);

// Launch counter of this library's kernels (read through flock_kernel_launches).
int flock_launch_fold_lsb(const void* in, size_t n_out, const uint64_t r[2], void* out, cudaStream_t st);
int flock_launch_zc_round0_skip(const void* a, const void* b, size_t n_pairs, const void* lag, void* A0, void* B0,
                                const void* eq_lo, const void* eq_hi, int lo_bits, void* partials, int grid,
                                cudaStream_t st);
// Zerocheck rounds 0..5 with the fixed-challenge eq factorisation
// (zc_round_grp_kernel): skip != 0 is round 0 from the bit rows in0, in1 (lag:
// the 64 skip Lagrange weights); otherwise in0, in1 are bound at rho. eq_lo
// covers the phi8 and lowest general variables (lo_bits), eq_hi the rest.
int flock_launch_zc_round_grp(const void* in0, const void* in1, size_t n_pairs, int skip, const uint64_t rho[2],
                              const void* lag, void* Aout, void* Bout, const void* eq_lo, const void* eq_hi,
                              int lo_bits, int a_bits, int m_bits, int m_mul, void* partials, int grid,
                              cudaStream_t st);
void flock_count_launch();
// Runs fn once per (current device, key), under a lock, so no thread passes
// before the first caller's fn has finished: per-device one-time work such as
// raising a kernel's shared-memory limit.
void flock_once_per_device(const void* key, void (*fn)());

// Hash-chain relation (chain.cu). g = [in || out] region folds of n_inst
// instances; W the shift-sumcheck weights; chain_round binds (bind != 0) the
// 2h-entry tables at r and writes per-block (q(1), q(inf)) partials of the
// h-entry tables; claim_basis adds c[p] eq(point, i) at word 128 i + p, p < 4.
int flock_launch_chain_fold_io(const void* z, size_t n_inst, const uint64_t e0[2], const uint64_t e1[2], void* g,
                               cudaStream_t st);
int flock_launch_chain_weights(const void* lo, const void* hi, int lo_bits, size_t n_inst, const uint64_t alpha[2],
                               void* W, cudaStream_t st);
int flock_chain_round_grid(size_t h);
int flock_launch_chain_round(void* W, void* g, size_t h, int bind, const uint64_t r[2], void* partials, int grid,
                             cudaStream_t st);
int flock_launch_chain_claim_basis(void* b, size_t n_inst, const void* lo, const void* hi, int lo_bits,
                                   const uint64_t c[8], cudaStream_t st);

// Benchmark inputs (inputs.cu): n records from SplitMix64 state `state0`.
int flock_launch_gen_inputs(uint64_t state0, size_t n, void* d_out, cudaStream_t st);

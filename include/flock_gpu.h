/*
 * flock_gpu.h - C ABI of the GB300 (sm_103a) prover for batched BLAKE3
 * compressions (Flock: R1CS over GF(2), zerocheck + lincheck + Ligerito PCS).
 *
 * Plain C types only: host pointers, device pointers (void*), sizes and
 * cudaStream_t passed as void*. Every function returns an int status
 * (FLOCK_OK = 0, negative on error) and never throws across the boundary.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the Layr-Labs/flock-challenge project root).
 */
#ifndef FLOCK_GPU_H
#define FLOCK_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FLOCK_PENDING = 1,      /* a served request is not finished yet (not an error) */
  FLOCK_OK = 0,
  FLOCK_ERR_SHAPE = -1,   /* size / shape outside the supported range */
  FLOCK_ERR_CUDA = -2,    /* a CUDA call failed */
  FLOCK_ERR_OOM = -3,     /* device allocation failed / over budget */
  FLOCK_ERR_ARG = -4,     /* null or inconsistent argument */
  FLOCK_ERR_CAPACITY = -5,/* output buffer too small */
  FLOCK_ERR_TIMEOUT = -6, /* a bounded wait or search gave up: a host wait passed the context's
                           wait limit (flock_set_wait_limit), or the grind's nonce range ran out */
  FLOCK_ERR_VERIFY = -7,  /* an internal consistency check failed */
  FLOCK_ERR_LIMIT = -8    /* size above the fixed limit of an entry point that allocates nothing */
};

/* One BLAKE3 compression input (112 bytes). Mirrors the reference tuple
 * `Compression = ([u32; 8], [u32; 16], u64, u32, u32)` of
 * crates/flock-prover/src/r1cs_hashes/blake3.rs:1087 and the benchmark's
 * RawCompression (benchmark-tools/common/src/lib.rs:1). */
typedef struct flock_compression {
  uint32_t cv[8];
  uint32_t m[16];
  uint64_t counter;
  uint32_t block_len;
  uint32_t flags;
} flock_compression;

typedef struct flock_ctx flock_ctx;

/* Library version string. */
const char* flock_version(void);

/* Number of CUDA kernels this library has launched in the process (all
 * contexts). No reference counterpart; used to count launches per proof. */
uint64_t flock_kernel_launches(void);

/* Threading: the library has no lock inside a context. A context (and the
 * buffers, stream and staging memory it owns) must be used by one host thread
 * at a time: give each thread its own context, or serialise the calls on a
 * shared one. Different contexts may run concurrently, also on one device.
 * The stage entry points without a context (flock_witness, flock_merkle_tree,
 * flock_generate_inputs) are thread-safe; flock_ntt_noalloc is thread-safe
 * only for calls whose work does not overlap on the GPU (see there). */

/* Create / destroy a device context bound to `device`. `hbm_budget` bounds the
 * device memory the context may hold (0 = no limit): a proof whose
 * flock_footprint_bytes exceeds it returns FLOCK_ERR_OOM.
 * Replaces the process-level setup of the reference worker
 * (benchmark-tools/worker/src/main.rs:45-57) and the Metal context of
 * crates/flock-core/src/gpu_commit.rs:1454-1478. */
int flock_create(int device, size_t hbm_budget, flock_ctx** out);
void flock_destroy(flock_ctx* ctx);

/* ---- Stage entry points on device buffers ------------------------------ */

/* Witness generation for 2^n_blocks_log compression slots (slots >= n are
 * the all-zero padding compression). d_in: n device records. Outputs
 * (device): z, a, b each 2^(n_blocks_log+14)/8 bytes in the packed F128
 * layout; d_a/d_b may both be null; stripe 2^(n_blocks_log+14)/8 bytes in the
 * lincheck byte-stripe layout, may be null.
 * Replaces generate_witness_with_ab_packed_and_lincheck
 * (crates/flock-prover/src/r1cs_hashes/blake3.rs:2948-3180). */
int flock_witness(const flock_compression* d_in, size_t n, int n_blocks_log, void* d_z, void* d_a,
                  void* d_b, void* d_stripe, void* stream);

/* Interleaved additive NTT (LCH novel basis, standard subspace {1, x, ...})
 * in place on d_data[pos * num_ntts + lane], 2^log_d positions, from layer
 * start_layer. Replaces AdditiveNttF128::forward_transform_interleaved_from_layer
 * (crates/flock-core/src/ntt/additive_ntt_f128.rs:599-622). */
int flock_ntt(flock_ctx* ctx, void* d_data, int log_d, int log_num_ntts, int start_layer, void* stream);

/* The NTT autotuner's choice for a transform shape (2^log_d positions x
 * 2^log_lanes lanes from start_layer) on `device`, or -1 if that shape has not
 * run yet: the multiply-pass shape (0, 1, 2: 4, 8 or 16 positions per thread;
 * 3: the deep-table pass, the last three layers of a 64-lane code through
 * tables of its narrow twiddles' products) and the end layer of the
 * byte-table passes (the upper layers run as
 * two-layer table passes while a block holds at least 2^k position-quads x
 * lanes, k tuned among 8, 9, 10; the layers from the end layer on run as
 * multiply passes). The first flock_ntt / commit / proof of a shape times the
 * candidates on a scratch buffer and keeps the fastest; FLOCK_NTT_TUNE=0 in the
 * environment disables tuning (k = 9, shape 1). No reference counterpart. */
int flock_ntt_tuned_variant(int device, int log_d, int log_lanes, int start_layer);
int flock_ntt_tuned_table_end(int device, int log_d, int log_lanes, int start_layer);

/* The narrow twiddle classes of a transform of 2^log_d positions: bytes 0..3
 * are the first layers from which every twiddle is below 2^32, 2^40, 2^64
 * and 2^72 (log_d where no layer qualifies). The multiply passes take 4
 * (below 2^32), 4 plus a shifted copy per higher bit (below 2^40), 6 (below
 * 2^64), 6 plus shifted copies (below 2^72) or 9 (otherwise) 32x32
 * carry-less pieces per product. Host arithmetic only (no device call);
 * FLOCK_ERR_ARG outside 1 <= log_d <= 40. No reference counterpart. */
int flock_ntt_twiddle_classes(int log_d);

/* The Merkle autotuner's choice for a tree shape (n_leaves leaves of
 * leaf_bytes) on `device`, or -1 if that shape has not run yet (or has fewer
 * than 2^12 leaves, which are never tuned): how many parent levels (0..2) the
 * leaf kernel folds in by warp shuffles before the parent kernels take over.
 * The first tree of a shape is built once per candidate and timed (every build
 * writes the same tree); FLOCK_MERKLE_TUNE=0 in the environment disables
 * tuning (no fused levels). No reference counterpart. */
int flock_merkle_tuned_levels(int device, size_t n_leaves, size_t leaf_bytes);

/* Largest log_d flock_ntt_noalloc accepts (2^16 positions per transform). */
#define FLOCK_NTT_NOALLOC_MAX_LOG_D 16

/* flock_ntt for callers that cannot allocate device memory (a host framework
 * that owns the GPU's memory through its own pool, or code running where
 * cudaMalloc is not allowed). No counterpart in the reference: it exists for
 * those callers only. Same transform, arguments and output as flock_ntt on
 * the current device, without a context, for 3 <= log_num_ntts <= 10 (8 to
 * 1024 interleaved transforms; other counts return FLOCK_ERR_SHAPE). The
 * twiddle table lives in a fixed 1 MiB device array of the library (held on
 * every GPU that loads it until exit); log_d above FLOCK_NTT_NOALLOC_MAX_LOG_D
 * returns FLOCK_ERR_LIMIT. The first call in a CUDA context (once per device,
 * unless the context is reset) looks up that array's address, so make it
 * before any stream capture. Calls share the array: calls whose work overlaps
 * on the GPU race. It runs only the generic multiply passes (no byte-table
 * passes, no tuned pass shape), so it is slower than flock_ntt. Calls no
 * cudaMalloc, cudaFree or other allocating routine. */
int flock_ntt_noalloc(void* d_data, int log_d, int log_num_ntts, int start_layer, void* stream);

/* Flat BLAKE3 Merkle tree (leaves first, root last; 2*n_leaves-1 nodes of 32
 * bytes) over n_leaves (a power of two) equal leaves of leaf_bytes: a
 * multiple of 16 up to 1024 (one BLAKE3 chunk), or 2048, 3072 or 4096 (whole
 * chunks); other sizes return FLOCK_ERR_SHAPE.
 * Replaces merkle::merkle_tree (crates/flock-core/src/merkle.rs:733-765). */
int flock_merkle_tree(const void* d_data, size_t n_leaves, size_t leaf_bytes, void* d_tree, void* stream);

/* PCS commit of a packed witness d_z (2^(m-7) F128): replicate into
 * 2^log_inv_rate blocks, NTT from layer log_inv_rate, Merkle over one leaf
 * per position. d_codeword: 2^(m-7+log_inv_rate) F128; d_tree:
 * 2*2^(m-7-log_batch_size+log_inv_rate)-1 nodes. root (host, 32 bytes).
 * Replaces pcs::commit (crates/flock-core/src/pcs/commit.rs:250-289) and the
 * Metal offload seam commit_l0_or_fallback (crates/flock-core/src/gpu_commit.rs:1467). */
int flock_commit(flock_ctx* ctx, const void* d_z, int m, int log_inv_rate, int log_batch_size,
                 void* d_codeword, void* d_tree, uint8_t root[32], void* stream);

/* ---- Full proof --------------------------------------------------------- */

/* Builds (and caches) the setup for proofs of n_blocks compressions: the
 * statement digest of the block R1CS (crates/flock-core/src/r1cs.rs:343-365)
 * and the device copies of the base matrices. Replaces Blake3Setup::new
 * (crates/flock-prover/src/r1cs_hashes/blake3.rs:3295-3347). Optional: the
 * first flock_prove does the same work. */
int flock_setup(flock_ctx* ctx, size_t n_blocks);

/* Proves n host compressions (padded to 2^max(3, ceil(log2 n)) slots with the
 * all-zero compression) and writes the serialized proof bundle
 * ("FLOCK" 0x04 0x02 + bincode, crates/flock-prover/src/proof_io.rs:161-208)
 * to out. *len receives the size; FLOCK_ERR_CAPACITY when cap is too small.
 * Replaces Blake3Setup::prove_fast + R1csProofBundleLigerito::to_bytes
 * (blake3.rs:3405-3480, proof_io.rs:161). Transcript domain "flock-bench-v0",
 * BLAKE3 Merkle/Fiat-Shamir, Fast profile, rate 1/2, 64 lanes. */
int flock_prove(flock_ctx* ctx, const flock_compression* in, size_t n, uint8_t* out, size_t cap, size_t* len);

/* Benchmark inputs: the 2^log2_size compressions the reference derives from
 * `seed` (generate_compressions, benchmark-tools/common/src/lib.rs:20-33),
 * generated on the device into d_out (2^log2_size records). */
int flock_generate_inputs(uint32_t log2_size, uint64_t seed, void* d_out, void* stream);

/* Seed to proof bytes: generates the inputs of `seed` on the device and
 * proves them (the reference worker's timed path, benchmark-tools/worker/src/
 * main.rs:66-79: generate_compressions + prove_fast + to_bytes).
 * 8 <= log2_size <= 21. */
int flock_prove_seed(flock_ctx* ctx, uint32_t log2_size, uint64_t seed, uint8_t* out, size_t cap, size_t* len);

/* As flock_prove, with the n input records already in device memory (d_in).
 * No reference counterpart (the reference's inputs live in host memory). */
int flock_prove_device(flock_ctx* ctx, const flock_compression* d_in, size_t n, uint8_t* out, size_t cap,
                       size_t* len);

/* The CUDA stream (cudaStream_t) the context's prover launches on, for
 * event timing by the caller. No reference counterpart. */
void* flock_stream(flock_ctx* ctx);

/* Host wall time (ms) of the phases of the last proof: setup, commit,
 * zerocheck round 1, zerocheck rounds, lincheck, ring switch, Ligerito,
 * serialization (first n entries). No reference counterpart (the reference's
 * FLOCK_PHASE_TIMING prints, crates/flock-prover/src/prover.rs:958-1216). */
int flock_last_phase_times(const flock_ctx* ctx, double* ms, int n);

/* The host's waits for the context's stream in each phase of the last proof
 * (same phase order, first n entries): how many, and the host time spent
 * blocked in them (ms). A phase's wall time minus its blocked time is the
 * host's own work (launches, transcript, host rounds). No reference
 * counterpart (measurement only). */
int flock_last_host_waits(const flock_ctx* ctx, uint64_t* waits, double* blocked_ms, int n);

/* CUDA-event timing of the main kernels of every proof on this context, on
 * the prover's own stream (enable != 0 turns it on; off by default), and
 * the device time (ms) of each span of the last proof: witness, L0 NTT,
 * L0 Merkle tree, zerocheck round 1 (first n entries; 0 while timing is off).
 * No reference counterpart (measurement only). */
int flock_kernel_timing(flock_ctx* ctx, int enable);
int flock_last_kernel_times(const flock_ctx* ctx, double* ms, int n);

/* Bounded waits. With limit_ms > 0, every host wait of this context's later
 * prove, prove_seed, prove_device, prove_challenger, chain and verify calls
 * (a round's partial sums, a grind result, a Merkle root, the start-of-call
 * drain of the previous call's work) polls the context's stream and gives
 * up after limit_ms: the call then returns FLOCK_ERR_TIMEOUT and writes no
 * output. The work the call had already queued keeps running on the GPU;
 * the context's next call waits for it first (under the same limit), so
 * the context stays usable. The limit bounds each wait, not a whole call.
 * 0 (the default): unbounded stream synchronisation. FLOCK_ERR_ARG for a
 * negative or NaN limit. The reference has no counterpart: its GPU waits
 * spin for a bounded budget and then block in waitUntilCompleted without a
 * deadline (crates/flock-core/src/gpu_commit.rs:1250-1257), and on a GPU
 * error it falls back to the CPU (:1462-1465). */
int flock_set_wait_limit(flock_ctx* ctx, double limit_ms);

/* ---- Verification -------------------------------------------------------- */

/* Verifies a serialized proof bundle: *accepted = 1 if it is a valid proof of
 * its statement (the batch-of-BLAKE3-compressions R1CS of its m), 0
 * otherwise (malformed bytes included). The transcript replay and the
 * sumcheck, Merkle and proof-of-work checks run on the host; the lincheck
 * matrix fold, the ring-switch combined basis and the Ligerito residual run
 * on the device. Replaces R1csProofBundleLigerito::from_bytes +
 * verifier::verify_ligerito (crates/flock-prover/src/proof_io.rs:161-208,
 * crates/flock-core/src/verifier.rs). */
int flock_verify(flock_ctx* ctx, const uint8_t* proof, size_t len, int* accepted);

/* flock_verify over count proofs (accepted[i] per proof). The reference's
 * verifier checks one bundle per call (benchmark-tools/harness verification
 * of each trial). */
int flock_verify_batch(flock_ctx* ctx, size_t count, const uint8_t* const* proofs, const size_t* lens,
                       int* accepted);

/* ---- The prove_fast seam: a caller-owned transcript and the claims ------- */

/* A Fiat-Shamir transcript on the host: FsChallenger::with_hash(domain,
 * HashKind::Blake3) (crates/flock-core/src/challenger.rs:183-438), i.e. the
 * `&mut impl Challenger` that Blake3Setup::prove_fast takes
 * (crates/flock-prover/src/r1cs_hashes/blake3.rs:3405-3409). F128 values are
 * {lo, hi} little-endian u64 pairs. A handle is not thread-safe: use one per
 * thread or serialise the calls on it. */
typedef struct flock_transcript flock_transcript;

/* FsChallenger::with_hash(domain, Blake3) (challenger.rs:214-240). */
int flock_transcript_create(const uint8_t* domain, size_t domain_len, flock_transcript** out);
/* Challenger::fork (challenger.rs:95-110): an independent copy of the state. */
int flock_transcript_fork(const flock_transcript* t, flock_transcript** out);
void flock_transcript_destroy(flock_transcript* t);
/* Challenger::observe_label / observe_f128 / observe_f128_slice /
 * observe_bytes (challenger.rs:34-60, FsChallenger's byte encoding). */
int flock_transcript_observe_label(flock_transcript* t, const uint8_t* label, size_t len);
int flock_transcript_observe_f128(flock_transcript* t, const uint64_t value[2]);
int flock_transcript_observe_f128_slice(flock_transcript* t, const uint64_t* values, size_t n);
int flock_transcript_observe_bytes(flock_transcript* t, const uint8_t* bytes, size_t len);
/* Challenger::sample_f128, and FsChallenger's sample_f128_vec (one squeeze of
 * 16 n bytes, not n single samples). */
int flock_transcript_sample_f128(flock_transcript* t, uint64_t out[2]);
int flock_transcript_sample_f128_vec(flock_transcript* t, size_t n, uint64_t* out);

/* Most outer coordinates a claim holds (m - 14 <= 21 for m <= 35). */
#define FLOCK_CLAIM_MAX_OUTER 24

/* ZClaim: z_hat(point) = value, point = QuirkyPoint { z_skip, x_inner_rest,
 * x_outer } (crates/flock-core/src/proof.rs:26-29, lincheck.rs:418-426) in the
 * BLAKE3 relation's RowMajor layout (crates/flock-core/src/r1cs.rs:289-334):
 * 8 inner coordinates, n_outer = m - 14 outer ones. */
typedef struct flock_zclaim {
  uint64_t z_skip[2];
  uint64_t x_inner_rest[8][2];
  uint64_t x_outer[FLOCK_CLAIM_MAX_OUTER][2];
  uint32_t n_outer;
  uint64_t value[2];
} flock_zclaim;

/* R1csClaim { ab, c } (crates/flock-core/src/proof.rs:36-45): ab from
 * lincheck, c from the zerocheck's extracted C evaluation. */
typedef struct flock_r1cs_claim {
  flock_zclaim ab, c;
} flock_r1cs_claim;

/* Blake3Setup::prove_fast(&self, &[Compression], &mut impl Challenger) ->
 * (R1csProofLigerito, Commitment, R1csClaim) (blake3.rs:3405-3409). Proves n
 * compressions (host records, or device records when in_on_device != 0) as
 * flock_prove does, but continues the caller's transcript `tr` (its domain
 * and whatever it has absorbed) instead of a fresh "flock-bench-v0" one, and
 * leaves it advanced past the proof, as the reference leaves the challenger.
 * Outputs: out = the proof bundle (the Commitment and R1csProofLigerito
 * serialized as R1csProofBundleLigerito::to_bytes, proof_io.rs:161-208),
 * root (32 bytes, may be null) = the commitment root, claim (may be null) =
 * the R1csClaim. On any status other than FLOCK_OK, `tr` is unchanged: with
 * FLOCK_ERR_CAPACITY (*len set) a second call with a larger buffer and the
 * same transcript returns the same proof. */
int flock_prove_challenger(flock_ctx* ctx, const flock_compression* in, size_t n, int in_on_device,
                           flock_transcript* tr, uint8_t* out, size_t cap, size_t* len, uint8_t root[32],
                           flock_r1cs_claim* claim);

/* flock_verify continuing the caller's transcript (the verifier side of the
 * same seam, crates/flock-core/src/verifier.rs); `tr` is advanced only when
 * the proof is accepted. */
int flock_verify_challenger(flock_ctx* ctx, const uint8_t* proof, size_t len, flock_transcript* tr, int* accepted);

/* ---- Hash chains ---------------------------------------------------------- */

/* Proves that n = 2^k compressions (2^8 <= n <= 2^21) form a sequential chain,
 * in[i + 1].cv == the first 8 output words of compress(in[i]), with public
 * endpoints cv_0 = in[0].cv and cv_last = the first 8 output words of
 * compress(in[n - 1]): the R1CS proof of the n compressions plus the shift
 * sumcheck, opened together with one PCS opening. Writes the chain bundle
 * ("FLOCK" 4 3, hash kind, commitment, proof, endpoint bits). A broken chain
 * still yields a bundle; the verifier rejects it. domain NULL =
 * "flock_chain-cli". Replaces Blake3Setup::prove_chain
 * (crates/flock-prover/src/r1cs_hashes/blake3.rs:3785-3805) and
 * ChainProofBundleLigerito::to_bytes (crates/flock-prover/src/proof_io.rs:486-493)
 * as the flock_chain CLI calls them (crates/flock-prover/src/bin/flock_chain.rs:222-262). */
int flock_prove_chain(flock_ctx* ctx, const flock_compression* in, size_t n, const char* domain, uint8_t* out,
                      size_t cap, size_t* len);

/* Verifies a chain bundle under domain (NULL = "flock_chain-cli"); *accepted
 * as in flock_verify. Replaces ChainProofBundleLigerito::from_bytes +
 * Blake3Setup::verify_chain (proof_io.rs:494-497, blake3.rs:3807-3830). */
int flock_verify_chain(flock_ctx* ctx, const uint8_t* bundle, size_t len, const char* domain, int* accepted);

/* Host-side honest chain as the flock_chain CLI builds it
 * (crates/flock-prover/src/bin/flock_chain.rs:180-196, :222-245): message words
 * are the low 32 bits of SplitMix64(seed) draws, counter 0, block_len 64,
 * flags 0, each cv the previous output; cv0 NULL = the BLAKE3 IV. Sequential
 * by nature (each cv depends on the previous compression). */
int flock_chain_inputs(size_t steps, uint64_t seed, const uint32_t* cv0, flock_compression* out);

/* ---- Batched and served proving ---------------------------------------- */

/* Device bytes one prover holds for a proof of 2^log2_size compressions (the
 * admission estimate of the server and of hbm_budget). No reference
 * counterpart. */
size_t flock_footprint_bytes(uint32_t log2_size);

typedef struct flock_server flock_server;

/* A proof server on `device` with n_workers concurrent provers (each its own
 * CUDA stream and resident buffers). Requests are admitted, in arrival order
 * where they fit, while the workers' device memory stays within hbm_budget
 * (0 = no limit); requests that arrive while others run start as soon as a
 * worker and memory are free, so their kernels overlap on the device.
 * Replaces the reference's worker-per-proof serving loop
 * (benchmark-tools/worker/src/main.rs:45-90) with continuous batching on one
 * GPU. */
int flock_server_create(int device, size_t hbm_budget, int n_workers, flock_server** out);
/* Finishes the queued requests, then stops the workers and frees the device. */
void flock_server_destroy(flock_server* s);
/* Queue a proof of the 2^log2_size benchmark inputs of `seed` (8..21), as
 * flock_prove_seed; *id identifies the request. FLOCK_ERR_OOM when the proof
 * alone exceeds the budget. */
int flock_server_submit_seed(flock_server* s, uint32_t log2_size, uint64_t seed, uint64_t* id);
/* Queue a proof of n host compressions (copied), as flock_prove. */
int flock_server_submit(flock_server* s, const flock_compression* in, size_t n, uint64_t* id);
/* FLOCK_PENDING while running; else the request's status, with the proof
 * copied to out (FLOCK_ERR_CAPACITY, *len set, keeps the proof for a retry).
 * A collected request is forgotten. */
int flock_server_poll(flock_server* s, uint64_t id, uint8_t* out, size_t cap, size_t* len);
/* As flock_server_poll, blocking until the request is finished. */
int flock_server_wait(flock_server* s, uint64_t id, uint8_t* out, size_t cap, size_t* len);
/* Queue and run times (ms) of a finished, not yet collected request. */
int flock_server_request_times(flock_server* s, uint64_t id, double* queue_ms, double* run_ms);
/* Device bytes the server's workers hold or have reserved. */
size_t flock_server_reserved_bytes(flock_server* s);
/* Batched form: proofs of count (size, seed) pairs through the server's
 * workers (largest first), written to out back to back in input order with
 * lens[i] their sizes. Each proof equals flock_prove_seed's for that pair.
 * No single reference counterpart (the reference proves one bundle per
 * worker run). */
int flock_prove_batch(flock_server* s, size_t count, const uint32_t* log2_sizes, const uint64_t* seeds, uint8_t* out,
                      size_t cap, size_t* lens);

#ifdef __cplusplus
}
#endif

#endif /* FLOCK_GPU_H */

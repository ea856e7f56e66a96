// Full-proof orchestration (prover.cu).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/flock_gpu.h"

struct ProverState;
namespace fs {
class Transcript;
}

// Host wall time of each phase of the last proof, in milliseconds, and the
// host's waits for the stream in each phase (count, and time blocked in them).
struct FlockPhaseTimes {
  double setup_ms = 0, commit_ms = 0, zc_round1_ms = 0, zc_rounds_ms = 0, lincheck_ms = 0, ring_switch_ms = 0,
         ligerito_ms = 0, serialize_ms = 0;
  uint64_t waits[8] = {};
  double blocked_ms[8] = {};
};

// A hash-chain proof (Blake3Setup::prove_chain, crates/flock-prover/src/r1cs_hashes/blake3.rs:3785-3805):
// the transcript domain and the public endpoints written into the bundle.
struct ChainReq {
  const char* domain = "flock_chain-cli";
  uint32_t cv0[8] = {0}, cv_last[8] = {0};
};

ProverState* flock_prover_create(int device);
void flock_prover_destroy(ProverState* s);
// Proves n host compressions in 2^n_log slots; `out` receives the wire bytes.
// With `chain`, the n = 2^n_log compressions form a cv chain and `out` is the
// chain bundle (ChainProofBundleLigerito) instead of the R1CS bundle.
// With `tr`, the proof continues the caller's transcript instead of a fresh
// one of the benchmark domain, and leaves it advanced (only on success);
// `claim` (optional) receives the R1CS claim the proof opens.
int flock_prover_prove(ProverState* s, const flock_compression* in, size_t n, int n_log, std::vector<uint8_t>& out,
                       bool input_on_device = false, const ChainReq* chain = nullptr, fs::Transcript* tr = nullptr,
                       flock_r1cs_claim* claim = nullptr);
cudaStream_t flock_prover_stream(const ProverState* s);
// Proofs from now on run on the prover's high-priority stream (high) or its
// normal one: the device dispatches blocks of high-priority kernels first.
// Waits for the prover's outstanding work when the stream changes.
void flock_prover_set_priority(ProverState* s, bool high);
// Generates the 2^log2 benchmark inputs of `seed` on the device, then proves them.
int flock_prover_prove_seed(ProverState* s, int log2, uint64_t seed, std::vector<uint8_t>& out);
const FlockPhaseTimes& flock_prover_times(const ProverState* s);
// CUDA-event timing of the main kernels of each proof (off by default) and
// the spans of the last proof in ms: witness, L0 NTT, L0 Merkle tree,
// zerocheck round 1.
int flock_prover_set_timing(ProverState* s, bool on);
int flock_prover_kernel_times(const ProverState* s, double* ms, int n);
// Bounds every host wait of the state's later calls by limit_ms (0: no
// bound): a wait that passes it makes the call return FLOCK_ERR_TIMEOUT.
int flock_prover_set_wait_limit(ProverState* s, double limit_ms);
// Device bytes the state holds (its buffers grow to the largest proof seen).
size_t flock_prover_reserved_bytes(const ProverState* s);
// Frees the state's device buffers (after its stream is idle); the next proof
// allocates them again.
void flock_prover_trim(ProverState* s);
// Verifies a serialized proof bundle (host transcript and checks, device
// kernels for the witness-size parts); *accepted = 1 when it verifies, `why`
// (optional) names the failed check. Returns a CUDA error code only when the
// device work fails.
#include <string>
// With `tr`, the replay continues the caller's transcript (advanced only when
// the proof is accepted).
int flock_prover_verify(ProverState* s, const uint8_t* data, size_t len, int* accepted, std::string* why,
                        fs::Transcript* tr = nullptr);
// Verifies a chain bundle (verify_chain, blake3.rs:3807-3830) under `domain`.
int flock_prover_verify_chain(ProverState* s, const uint8_t* data, size_t len, const char* domain, int* accepted,
                              std::string* why);

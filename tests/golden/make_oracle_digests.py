"""Regenerates the oracle proof fixtures in this folder from the CPU oracle.

Usage: python tests/golden/make_oracle_digests.py

Needs no reference checkout: it builds and runs the oracle (oracle/, test
infrastructure) and reads the reference-held pins from reference_pins.json
(written by make_golden.py).

canary_2e18.json     the oracle's proof of the ranked canary input (2^18
                     compressions, crates/flock-prover/src/r1cs_hashes/
                     blake3.rs:4910-4930): its length, which must equal the
                     reference's EXPECTED_PROOF_BYTES, its BLAKE3 and SHA-256,
                     and the oracle verifier's verdict.
oracle_digests.json  BLAKE3 digests and lengths of the oracle's proofs of the
                     benchmark inputs (benchmark-tools/common/src/lib.rs:20-33)
                     at 2^14 compressions for seeds 0..4 and the worker's
                     warm-up seed, and at 2^18 for seeds 0 and 1.

A 2^18 oracle proof takes one to two minutes on eight x86 cores.
"""
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib as O  # noqa: E402

CONFIG0_SEEDS = [0, 1, 2, 3, 4]
RANKED_SEEDS = [0, 1]


def proof_record(log2, seed, canary=False):
    t = time.time()
    p = O.prove(O.compressions(log2, seed, canary=canary), log2)
    ok, why = O.verify(p, 14 + log2)
    if not ok:
        raise SystemExit(f"oracle verifier rejected its own proof (2^{log2}, seed {seed}): {why}")
    print(f"2^{log2} seed {seed:#x}{' canary' if canary else ''}: {len(p)} bytes, {time.time() - t:.1f} s",
          flush=True)
    return p


def main():
    pins = json.load(open(os.path.join(HERE, "reference_pins.json")))
    canary = proof_record(18, 0, canary=True)
    if len(canary) != pins["canary_expected_proof_bytes"]:
        raise SystemExit(f"oracle canary proof is {len(canary)} bytes, the reference pins "
                         f"{pins['canary_expected_proof_bytes']}")
    json.dump({"n_blocks_log": 18,
               "input": "canary: SplitMix64 seeded 0xC0FFEEBEEF ^ 2^18, per op cv[8], m[16], counter = one u32 "
                        "draw, block_len 64, flags 11 (crates/flock-prover/src/r1cs_hashes/blake3.rs:4910-4930)",
               "reference_expected_proof_bytes": pins["canary_expected_proof_bytes"],
               "reference_source": pins["canary_source"],
               "oracle_proof_bytes": len(canary),
               "oracle_proof_blake3": O.b3_hash(canary).hex(),
               "oracle_proof_sha256": hashlib.sha256(canary).hexdigest(),
               "oracle_verifier": "accepted"},
              open(os.path.join(HERE, "canary_2e18.json"), "w"), indent=1)
    out = {"domain": "flock-bench-v0", "generator": "benchmark-tools/common/src/lib.rs:20-33", "proofs": []}
    for log2, seeds in [(14, CONFIG0_SEEDS + [pins["worker_warmup_seed"]]), (18, RANKED_SEEDS)]:
        for seed in seeds:
            p = proof_record(log2, seed)
            out["proofs"].append({"log2": log2, "seed": seed, "bytes": len(p), "blake3": O.b3_hash(p).hex()})
    json.dump(out, open(os.path.join(HERE, "oracle_digests.json"), "w"), indent=1)
    print("wrote canary_2e18.json, oracle_digests.json")


if __name__ == "__main__":
    main()

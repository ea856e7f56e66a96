"""Command-line prover: seed -> proof bundle on one GPU.

python -m flock_challenge_gb300.cli --log2 18 --seed 42 [--repeat 2] [--out proof.bin] [--times] [--chain]

Mirrors the reference worker's timed path (benchmark-tools/worker/src/main.rs:
generate_compressions(log2, seed) -> Blake3Setup::prove_fast -> to_bytes).
With --repeat R the same seed is proven R times in one process (the first proof
is the warm-up, as in the reference worker) and each proof's time is printed.
With --chain the proof is the hash-chain bundle of 2^log2 linked compressions
built as `flock_chain prove --hash blake3 --steps 2^log2 --seed S` builds them
(crates/flock-prover/src/bin/flock_chain.rs:222-262).
"""
import argparse
import sys
import time

from . import Blake3Setup, chain_inputs


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--log2", type=int, default=18)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--out", default=None)
    ap.add_argument("--times", action="store_true", help="print per-phase host times of the last proof")
    ap.add_argument("--chain", action="store_true", help="prove a hash chain (flock_prove_chain)")
    a = ap.parse_args(argv)
    setup = Blake3Setup(1 << a.log2, device=a.device)
    blocks = chain_inputs(1 << a.log2, a.seed) if a.chain else None
    proof = None
    for i in range(a.repeat):
        t = time.perf_counter()
        proof = setup.prove_chain(blocks) if a.chain else setup.prove_seed(a.seed)
        dt = time.perf_counter() - t
        print(f"proof {i}: {len(proof)} bytes in {dt * 1e3:.2f} ms", flush=True)
    if a.times:
        print(" ".join(f"{k}={v:.2f}ms" for k, v in setup.phase_times().items()))
    if a.out:
        with open(a.out, "wb") as f:
            f.write(proof)
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Regenerates the golden fixtures in this folder from the reference sources.

Usage: python tests/golden/make_golden.py REFERENCE_ROOT

REFERENCE_ROOT is the root of a Layr-Labs/flock-challenge checkout (required).
The fixtures are committed so the tests never read the reference at run time.

phi8.json          PHI_8_TABLE of crates/flock-core/src/field/phi8.rs:18-1040
                   (the GF(2^8) -> GF(2^128) embedding, 256 entries as [lo, hi]).
ghash_kat.json     the GHASH known-answer identities of
                   crates/flock-core/src/field/gf2_128.rs:378-405.
layout.json        the BLAKE3 witness layout constants asserted at
                   crates/flock-prover/src/r1cs_hashes/blake3.rs:4334-4350.
reference_pins.json  the canary's pinned proof length EXPECTED_PROOF_BYTES
                   (blake3.rs:4914) and the worker's warm-up seed
                   (benchmark-tools/worker/src/main.rs:29); make_oracle_digests.py
                   checks the oracle's canary proof against the former.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    raise SystemExit(__doc__)
ref = sys.argv[1]
here = os.path.dirname(os.path.abspath(__file__))

src = open(os.path.join(ref, "crates/flock-core/src/field/phi8.rs")).read()
body = src[src.index("PHI_8_TABLE"):src.index("];")]
pairs = re.findall(r"lo:\s*(0x[0-9a-fA-F]+),\s*hi:\s*(0x[0-9a-fA-F]+)", body)
assert len(pairs) == 256, len(pairs)
json.dump([[int(lo, 16), int(hi, 16)] for lo, hi in pairs], open(os.path.join(here, "phi8.json"), "w"))

# The KAT block of gf2_128.rs: pairs of operands and expected products.
gf = open(os.path.join(ref, "crates/flock-core/src/field/gf2_128.rs")).read()
assert "x · x^127" in gf and "x^64 · x^64" in gf
kat = [
    # [a_lo, a_hi, b_lo, b_hi, out_lo, out_hi] from the asserts at :378-405
    [2, 0, 0, 1 << 63, 0x87, 0],
    [2, 0, 1 << 63, 0, 0, 1],
    [0, 1, 0, 1, 0x87, 0],
    [2, 0, 2, 0, 4, 0],
]
json.dump(kat, open(os.path.join(here, "ghash_kat.json"), "w"))

b3 = open(os.path.join(ref, "crates/flock-prover/src/r1cs_hashes/blake3.rs")).read()
seg = b3[b3.index("fn layout_constants()"):]
seg = seg[:seg.index("}\n")]
layout = {k: int(v.replace("_", "")) for k, v in re.findall(r"assert_eq!\((\w+), ([0-9_]+)\)", seg)}
json.dump(layout, open(os.path.join(here, "layout.json"), "w"), indent=1, sort_keys=True)
canary = b3[b3.index("fn ranked_blake3_proof_canary()"):]
expected = int(re.search(r"EXPECTED_PROOF_BYTES: usize = ([0-9_]+);", canary).group(1).replace("_", ""))
worker = open(os.path.join(ref, "benchmark-tools/worker/src/main.rs")).read()
warm = int(re.search(r"generate_compressions\(log2_size, (0x[0-9A-Fa-f_]+)\)", worker).group(1).replace("_", ""), 16)
json.dump({"canary_expected_proof_bytes": expected,
           "canary_source": "crates/flock-prover/src/r1cs_hashes/blake3.rs:4914 EXPECTED_PROOF_BYTES",
           "worker_warmup_seed": warm,
           "worker_warmup_source": "benchmark-tools/worker/src/main.rs:29"},
          open(os.path.join(here, "reference_pins.json"), "w"), indent=1)
print("wrote", sorted(os.listdir(here)))

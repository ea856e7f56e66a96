"""Regenerates the golden fixtures in this folder from the reference sources.

Run once in a checkout that has the reference tree (path given as argv[1],
default /root/reference). The fixtures are committed so the tests never read
the reference at run time.

phi8.json          PHI_8_TABLE of crates/flock-core/src/field/phi8.rs:18-1040
                   (the GF(2^8) -> GF(2^128) embedding, 256 entries as [lo, hi]).
ghash_kat.json     the GHASH known-answer identities of
                   crates/flock-core/src/field/gf2_128.rs:378-405.
layout.json        the BLAKE3 witness layout constants asserted at
                   crates/flock-prover/src/r1cs_hashes/blake3.rs:4334-4350.
"""
import json
import os
import re
import sys

ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
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
print("wrote", sorted(os.listdir(here)))

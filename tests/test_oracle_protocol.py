"""Oracle protocol: prove -> verify round trips and tamper rejection.

Mirrors the reference's end-to-end tests (crates/flock-prover/src/r1cs_hashes/
blake3.rs:5006-5100 prove_verify roundtrips at m=22) and its mutation tests
(zerocheck.rs:1791-2112, lincheck.rs:2444 verify_rejects_mutations).
"""
import json
import os
import struct

import numpy as np
import pytest

import oracle_lib as O

N_LOG = 8  # m = 22, the smallest Ligerito-configured size


@pytest.fixture(scope="module")
def proof():
    blocks = O.compressions(N_LOG, 5)
    return O.prove(blocks, N_LOG)


def test_f8_extension_order_matches_reference_ntt():
    # ntt.rs:25-170 (inverse on S = {0..63}, forward on 64 + span{1..32}) puts
    # the evaluation at lambda = 64 + i in slot i: the Lambda node order the
    # verifier assumes (multilinear.rs:420-445, PHI_8_TABLE[64 + i]).
    rng = np.random.default_rng(3)
    for _ in range(8):
        row = int(rng.integers(0, 2**63)) | (int(rng.integers(0, 2)) << 63)
        assert np.array_equal(O.f8_extend(row, "ntt"), O.f8_extend(row, "lagrange"))


def test_roundtrip_accepts(proof):
    ok, why = O.verify(proof, 14 + N_LOG)
    assert ok, why
    assert proof[:7] == b"FLOCK\x04\x02"


def test_deterministic(proof):
    assert O.prove(O.compressions(N_LOG, 5), N_LOG) == proof


def test_ragged_input_pads_with_zero_compressions():
    blocks = O.compressions(N_LOG, 6)[:200]
    p = O.prove(blocks, N_LOG)
    ok, why = O.verify(p, 14 + N_LOG)
    assert ok, why


def _flip(p, off):
    b = bytearray(p)
    b[off] ^= 1
    return bytes(b)


@pytest.mark.parametrize("where", ["root", "zc_round1", "zc_final", "lc_round", "s_hat_v", "lig_open", "yr",
                                   "trailing", "truncated"])
def test_tamper_rejected(proof, where):
    hdr = 7
    root_off = hdr
    params_end = root_off + 32 + 3 * 8 + 2 * 4
    zc_r1 = params_end + 8  # first round1_ab element
    if where == "root":
        bad = _flip(proof, root_off + 3)
    elif where == "zc_round1":
        bad = _flip(proof, zc_r1 + 16 * 5)
    elif where == "zc_final":
        # final_a of the zerocheck: after round1_ab, round1_c and the rounds vector
        n_r = 14 + N_LOG - 6
        off = params_end + (8 + 64 * 16) * 2 + 8 + n_r * 32
        bad = _flip(proof, off)
    elif where == "lc_round":
        n_r = 14 + N_LOG - 6
        off = params_end + (8 + 64 * 16) * 2 + 8 + n_r * 32 + 48 + 8
        bad = _flip(proof, off)
    elif where == "s_hat_v":
        n_r = 14 + N_LOG - 6
        off = params_end + (8 + 64 * 16) * 2 + 8 + n_r * 32 + 48 + 8 + 8 * 32 + 8 + 64 * 16 + 8 + 8 + 40
        bad = _flip(proof, off)
    elif where == "lig_open":
        bad = _flip(proof, len(proof) // 2)
    elif where == "yr":
        bad = _flip(proof, len(proof) - 200)
    elif where == "trailing":
        bad = proof + b"\x00"
    else:
        bad = proof[:-1]
    ok, _ = O.verify(bad, 14 + N_LOG)
    assert not ok


def test_wrong_statement_size_rejected(proof):
    ok, _ = O.verify(proof, 14 + N_LOG + 1)
    assert not ok


@pytest.mark.slow
@pytest.mark.skipif(os.environ.get("FLOCK_SLOW_TESTS") != "1",
                    reason="one full 2^18 oracle proof (minutes on a few cores): set FLOCK_SLOW_TESTS=1")
def test_oracle_canary_proof_has_reference_length():
    # crates/flock-prover/src/r1cs_hashes/blake3.rs:4910-4939: the proof of the
    # ranked canary input is EXPECTED_PROOF_BYTES long (reference_pins.json,
    # extracted from the reference by make_golden.py), and its verifier accepts.
    gold = os.path.join(os.path.dirname(__file__), "golden")
    pins = json.load(open(os.path.join(gold, "reference_pins.json")))
    canary = json.load(open(os.path.join(gold, "canary_2e18.json")))
    p = O.prove(O.compressions(18, 0, canary=True), 18)
    assert len(p) == pins["canary_expected_proof_bytes"] == 437_551
    assert O.b3_hash(p).hex() == canary["oracle_proof_blake3"]
    ok, why = O.verify(p, 32)
    assert ok, why


def test_prove_with_transcript_matches_default_prove(proof):
    # a fresh transcript of the benchmark domain is the default proof; the
    # claim's points have the RowMajor shapes (8 inner, m - 14 outer)
    t = O.Transcript(b"flock-bench-v0")
    p, root, claim = O.prove_with(O.compressions(N_LOG, 5), N_LOG, t)
    assert p == proof and root == proof[7:39]
    assert len(claim["ab"]["x_inner_rest"]) == 8 and len(claim["c"]["x_outer"]) == N_LOG
    ok, why = O.verify_with(p, 14 + N_LOG, O.Transcript(b"flock-bench-v0"))
    assert ok, why
    ok, _ = O.verify_with(p, 14 + N_LOG, O.Transcript(b"another-domain"))
    assert not ok

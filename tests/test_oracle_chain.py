"""Oracle hash-chain relation (CPU): the shift MLE properties of
crates/flock-prover/src/chain.rs:565-610, the chain round trip and the three
rejections of crates/flock-prover/src/r1cs_hashes/blake3.rs:5173-5286
(honest chain accepts; broken link, wrong endpoint reject), the flock_chain
CLI's input generator, and the chain bundle's wire framing."""
import itertools
import random

import numpy as np
import pytest

import oracle_lib as O

ONE, ZERO = (1, 0), (0, 0)


def add(a, b):
    return (a[0] ^ b[0], a[1] ^ b[1])


def bits(v, n):
    return [ONE if (v >> j) & 1 else ZERO for j in range(n)]


def eq(a, b):
    acc = ONE
    for x, y in zip(a, b):
        acc = O.gf_mul(acc, add(add(ONE, x), y))
    return acc


def rand_f(rng):
    return (rng.getrandbits(64), rng.getrandbits(64))


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_shift_mle_boolean_is_successor(n):
    for a, b in itertools.product(range(1 << n), repeat=2):
        want = ONE if b == a + 1 else ZERO
        assert O.shift_mle(bits(a, n), bits(b, n)) == want, (a, b)


def test_shift_mle_top_has_no_successor():
    n = 4
    top = bits((1 << n) - 1, n)
    for b in range(1 << n):
        assert O.shift_mle(top, bits(b, n)) == ZERO


def test_shift_equals_shifted_eq():
    rng = random.Random(5)
    n = 5
    tau = [rand_f(rng) for _ in range(n)]
    for y in range(1, 1 << n):
        assert O.shift_mle(tau, bits(y, n)) == eq(tau, bits(y - 1, n)), y
    assert O.shift_mle(tau, bits(0, n)) == ZERO


def test_chain_inputs_link():
    blocks = O.chain_inputs(64, 0x1234)
    assert list(blocks[0]["cv"]) == [0x6A09E667, 0xBB67AE85, 0x3C6EF372, 0xA54FF53A,
                                     0x510E527F, 0x9B05688C, 0x1F83D9AB, 0x5BE0CD19]
    for i in range(63):
        b = blocks[i]
        assert (b["counter"], b["block_len"], b["flags"]) == (0, 64, 0)
        out = O.b3_compress(b["cv"], b["m"], 0, 64, 0)
        assert np.array_equal(out[:8], blocks[i + 1]["cv"])
    cv0 = np.arange(1, 9, dtype=np.uint32)
    assert np.array_equal(O.chain_inputs(4, 1, cv0)[0]["cv"], cv0)


@pytest.fixture(scope="module")
def honest():
    blocks = O.chain_inputs(256, 0xB35113E)
    return blocks, O.prove_chain(blocks)


def test_chain_roundtrip_accepts(honest):
    blocks, bundle = honest
    assert bundle[:7] == b"FLOCK\x04\x03"
    assert O.verify_chain(bundle) == (True, "ok")
    # endpoints: cv_0 and the last output, 256 bits each at the end of the bundle
    last = O.b3_compress(blocks[-1]["cv"], blocks[-1]["m"], 0, 64, 0)[:8]
    tail = np.frombuffer(bundle[-2 * 264:], np.uint8)
    assert int.from_bytes(bytes(tail[:8]), "little") == 256
    want0 = [(int(blocks[0]["cv"][i // 32]) >> (i % 32)) & 1 for i in range(256)]
    want1 = [(int(last[i // 32]) >> (i % 32)) & 1 for i in range(256)]
    assert list(tail[8:264]) == want0 and list(tail[272:]) == want1


@pytest.mark.parametrize("which", ["cv0", "cv_last"])
def test_wrong_endpoint_rejects(honest, which):
    _, bundle = honest
    b = bytearray(bundle)
    off = len(b) - 2 * 264 + 8 if which == "cv0" else len(b) - 256
    b[off + 3] ^= 1
    ok, why = O.verify_chain(bytes(b))
    assert not ok and why == "chain shift"


def test_broken_chain_rejects():
    blocks = O.chain_inputs(256, 0xB355)
    blocks["cv"][2] = np.arange(8, dtype=np.uint32) * 977  # instance 2 no longer follows instance 1
    ok, why = O.verify_chain(O.prove_chain(blocks))
    assert not ok


def test_wrong_domain_rejects(honest):
    _, bundle = honest
    assert not O.verify_chain(bundle, b"b3-chain")[0]


def test_chain_bundle_framing(honest):
    _, bundle = honest
    assert O.verify_chain(bundle[:-1])[1] == "malformed"
    assert O.verify_chain(bundle + b"\x00")[1] == "malformed"
    b = bytearray(bundle)
    b[-1] = 2  # a bool byte other than 0 / 1
    assert O.verify_chain(bytes(b))[1] == "malformed"
    b = bytearray(bundle)
    b[6] = 2  # R1CS flavor
    assert O.verify_chain(bytes(b))[1] == "malformed"

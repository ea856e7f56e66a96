"""Oracle pins: field KATs, phi8 table, layout constants, R1CS satisfaction."""
import json
import os

import numpy as np
import pytest

import oracle_lib as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_ghash_kats():
    # crates/flock-core/src/field/gf2_128.rs:378-405
    for a0, a1, b0, b1, o0, o1 in json.load(open(os.path.join(GOLD, "ghash_kat.json"))):
        assert O.gf_mul((a0, a1), (b0, b1)) == (o0, o1)


def test_product_paths_agree():
    # The oracle multiplies with PMULL on an Arm host with the crypto extension
    # (as the reference's aarch64 backend, crates/flock-core/src/field/gf2_128/
    # aarch64.rs:26-60) and with portable integer code elsewhere; both must
    # give the same products, KATs included.
    import ctypes
    L = O.lib()
    L.oracle_gf_crosscheck.restype = ctypes.c_size_t
    L.oracle_gf_crosscheck.argtypes = [ctypes.c_size_t, ctypes.c_uint64]
    L.oracle_gf_mul_portable.argtypes = [ctypes.c_void_p] * 3
    assert L.oracle_gf_crosscheck(200_000, 11) == 0
    for a0, a1, b0, b1, o0, o1 in json.load(open(os.path.join(GOLD, "ghash_kat.json"))):
        out = np.zeros(2, np.uint64)
        L.oracle_gf_mul_portable(O.ptr(np.array([a0, a1], np.uint64)), O.ptr(np.array([b0, b1], np.uint64)),
                                 O.ptr(out))
        assert (int(out[0]), int(out[1])) == (o0, o1)


def test_inverse_identities():
    # gf2_128.rs:408-430: a * a^-1 = 1, including top-bit inputs
    for a in [(0, 1 << 63), ((1 << 64) - 1, (1 << 64) - 1), (0, (1 << 64) - 1), (3, 0), (0x1234, 0x5678)]:
        assert O.gf_mul(a, O.gf_inv(a)) == (1, 0)


def test_mul_commutative_and_distributive():
    rng = np.random.default_rng(1)
    for _ in range(64):
        a, b, c = [tuple(int(x) for x in rng.integers(0, 2**63, 2, dtype=np.uint64)) for _ in range(3)]
        assert O.gf_mul(a, b) == O.gf_mul(b, a)
        bc = (b[0] ^ c[0], b[1] ^ c[1])
        ab, ac = O.gf_mul(a, b), O.gf_mul(a, c)
        assert O.gf_mul(a, bc) == (ab[0] ^ ac[0], ab[1] ^ ac[1])


def test_phi8_matches_reference_table_and_is_homomorphic():
    table = json.load(open(os.path.join(GOLD, "phi8.json")))
    for v in range(256):
        assert O.phi8(v) == tuple(table[v])
    rng = np.random.default_rng(2)
    for _ in range(200):
        a, b = (int(x) for x in rng.integers(0, 256, 2))
        assert O.phi8(O.lib().oracle_gf8_mul(a, b)) == O.gf_mul(O.phi8(a), O.phi8(b))


def test_layout_constants():
    lay = json.load(open(os.path.join(GOLD, "layout.json")))
    assert lay["USEFUL_BITS"] == 15409 and lay["Z_CONST_POS"] == 512 and lay["GS_BASE"] == 1153
    assert lay["G_STRIDE"] == 6 * 31 + 2 * 32 and lay["OUT_HI_BASE"] == 1153 + 56 * 250


def _unpack(words, n_blocks):
    return np.unpackbits(words.view(np.uint8), bitorder="little").reshape(n_blocks, 1 << 14)


@pytest.fixture(scope="module")
def mats():
    return O.matrices()


def _apply(bits, a_len, cols, offset):
    off = np.concatenate([[0], np.cumsum(a_len.astype(np.int64))]) + offset
    out = np.zeros(bits.shape, np.uint8)
    for r in range(1 << 14):
        c = cols[off[r]:off[r + 1]]
        if c.size:
            out[:, r] = bits[:, c].sum(axis=1) & 1
    return out


def test_honest_witness_satisfies_r1cs(mats):
    # blake3.rs:4421-4440: A*z = a, B*z = b and a & b = z (C = I)
    a_len, b_len, cols = mats
    blocks = O.compressions(3, 11)
    z, a, b, _ = O.witness(blocks[:5], 3)  # 3 padding slots
    zb, ab, bb = (_unpack(x, 8) for x in (z, a, b))
    Az = _apply(zb, a_len, cols, 0)
    Bz = _apply(zb, b_len, cols, int(a_len.astype(np.int64).sum()))
    assert np.array_equal(Az, ab)
    assert np.array_equal(Bz, bb)
    assert np.array_equal(ab & bb, zb)
    assert zb[:, 512].all()  # constant wire in every slot, padding included
    assert not zb[:, 15409:].any()


def test_mutated_witness_fails(mats):
    # blake3.rs:4442-4462: flipping one carry bit breaks a constraint
    a_len, b_len, cols = mats
    blocks = O.compressions(3, 12)
    z, a, b, _ = O.witness(blocks, 3)
    zb = _unpack(z, 8).copy()
    zb[0, 1153 + 5] ^= 1
    Az = _apply(zb, a_len, cols, 0)
    Bz = _apply(zb, b_len, cols, int(a_len.astype(np.int64).sum()))
    assert not np.array_equal(Az & Bz, zb)


def test_matrix_nnz_and_digest_stable():
    a_len, b_len, cols = O.matrices()
    assert cols.size == 21028097
    d28 = O.statement_digest(28)
    assert d28 == O.statement_digest(28)
    assert d28 != O.statement_digest(32)


def test_stripe_layout():
    blocks = O.compressions(4, 3)
    z, _, _, s = O.witness(blocks, 4, want_ab=False)
    zb = _unpack(z, 16)
    sb = np.unpackbits(s, bitorder="little").reshape(2, 1 << 14, 8)
    for j in range(16):
        assert np.array_equal(sb[j // 8, :, j % 8], zb[j])

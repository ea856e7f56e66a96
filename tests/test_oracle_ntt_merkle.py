"""Oracle pins for the additive NTT, BLAKE3 modes and the Merkle tree."""
import numpy as np

import oracle_lib as O


def gf(a, b):
    return O.gf_mul(a, b)


def add(a, b):
    return (a[0] ^ b[0], a[1] ^ b[1])


def test_ntt_is_novel_basis_evaluation():
    # additive_ntt_f128.rs:1-45: forward NTT maps novel-basis coefficients to
    # evaluations at the subspace points; position p holds the point whose
    # polynomial-basis encoding is p. X_j = prod_{i in bits(j)} What_i with
    # W_0(z) = z, W_i(z) = W_{i-1}(z) (W_{i-1}(z) + W_{i-1}(x^{i-1})).
    d = 4
    n = 1 << d
    rng = np.random.default_rng(5)
    coeffs = rng.integers(0, 2**63, (n, 2), dtype=np.uint64)
    out = O.ntt_interleaved(coeffs.reshape(-1), 1, 0).reshape(n, 2)

    def W(i, z):
        if i == 0:
            return z
        w = W(i - 1, z)
        return gf(w, add(w, W(i - 1, (1 << (i - 1), 0))))

    norms = [O.gf_inv(W(i, (1 << i, 0))) for i in range(d)]
    for p in range(n):
        z = (p, 0)
        what = [gf(W(i, z), norms[i]) for i in range(d)]
        acc = (0, 0)
        for j in range(n):
            xj = (1, 0)
            for i in range(d):
                if (j >> i) & 1:
                    xj = gf(xj, what[i])
            acc = add(acc, gf((int(coeffs[j, 0]), int(coeffs[j, 1])), xj))
        assert acc == (int(out[p, 0]), int(out[p, 1]))


def test_replicated_start_matches_zero_padded_transform():
    # pcs/commit.rs:451-473: r leading layers on [z, 0..] are copies
    rng = np.random.default_rng(6)
    lanes, log_msg, r = 4, 5, 2
    z = rng.integers(0, 2**63, (1 << log_msg) * lanes * 2, dtype=np.uint64)
    padded = np.zeros((1 << (log_msg + r)) * lanes * 2, np.uint64)
    padded[: z.size] = z
    full = O.ntt_interleaved(padded, lanes, 0)
    rep = np.tile(z, 1 << r)
    fast = O.ntt_interleaved(rep, lanes, r)
    assert np.array_equal(full, fast)


def test_blake3_single_block_hash_is_flags_11_compression():
    # The PoW pre-image (challenger.rs:1246-1296) and the benchmark inputs use
    # block_len 64 with flags CHUNK_START|CHUNK_END|ROOT = 11.
    rng = np.random.default_rng(7)
    data = rng.integers(0, 256, 64, dtype=np.uint8).tobytes()
    iv = [0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a, 0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19]
    words = np.frombuffer(data, "<u4")
    out = O.b3_compress(iv, words, 0, 64, 11)
    assert O.b3_hash(data) == out[:8].astype("<u4").tobytes()
    # XOF prefix equals the hash; XOF block k is the ROOT compression with counter k
    x = O.b3_xof(data, 128)
    assert x[:32] == O.b3_hash(data)
    assert x[:64] == out.astype("<u4").tobytes()
    assert x[64:] == O.b3_compress(iv, words, 1, 64, 11).astype("<u4").tobytes()


def test_leaf_cv_chunk_semantics():
    # merkle.rs:200-205 / gpu_commit.rs:2905-2919 (MSL mirror): a 1 KiB leaf is
    # 16 compressions, counter 0, CHUNK_START first, CHUNK_END last, no ROOT.
    rng = np.random.default_rng(8)
    data = rng.integers(0, 256, 1024, dtype=np.uint8).tobytes()
    cv = [0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a, 0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19]
    for b in range(16):
        flags = (1 if b == 0 else 0) | (2 if b == 15 else 0)
        cv = list(O.b3_compress(cv, np.frombuffer(data[64 * b:64 * b + 64], "<u4"), 0, 64, flags)[:8])
    assert O.leaf_cv(data) == np.array(cv, "<u4").tobytes()


def test_merkle_tree_flat_layout_and_multiproof():
    rng = np.random.default_rng(9)
    n, leaf = 16, 128
    data = rng.integers(0, 256, n * leaf, dtype=np.uint8)
    tree = O.merkle_tree(data, n)
    assert tree.shape == (2 * n - 1, 32)
    for i in range(n):
        assert tree[i].tobytes() == O.leaf_cv(data[i * leaf:(i + 1) * leaf].tobytes())

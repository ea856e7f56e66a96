"""GPU parity: witness, NTT, Merkle and PCS commit against the CPU oracle (bit-exact)."""
import numpy as np
import pytest

import flock_challenge_gb300 as F
import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(cuda_device):
    return F.Context(0)


def to_dev(arr):
    import torch
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1).copy()).cuda()


def host(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("n_log,n", [(3, 8), (3, 5), (5, 32), (6, 50), (9, 512), (10, 700)])
def test_witness_matches_oracle(cuda_device, n_log, n):
    blocks = O.compressions(max(n_log, 3), 1234 + n)[:n]
    z, a, b, s = F.generate_witness(to_dev(blocks), n, n_log)
    oz, oa, ob, os_ = O.witness(blocks, n_log)
    assert np.array_equal(host(z), oz.view(np.uint8))
    assert np.array_equal(host(a), oa.view(np.uint8))
    assert np.array_equal(host(b), ob.view(np.uint8))
    assert np.array_equal(host(s), os_)


def test_witness_z_only(cuda_device):
    blocks = O.compressions(6, 9)
    z, a, b, s = F.generate_witness(to_dev(blocks), 64, 6, want_ab=False, want_stripe=False)
    oz, _, _, _ = O.witness(blocks, 6, want_ab=False, want_stripe=False)
    assert a is None and s is None
    assert np.array_equal(host(z), oz.view(np.uint8))


# shapes whose upper layers run as byte-table passes (a block of the pass's
# first layer holds >= 2^9 quad-lanes): (7, 6, 1), (12, 6, 1), (13, 4, 3),
# (10, 6, 0), (9, 7, 2), (16, 6, 1), (14, 3, 2); (8, 3, 0) and (11, 4, 4) sit
# exactly at the cutoff (one table pass, then multiply passes). (12, 3, 1)
# puts layer 8, whose twiddles are below 2^65, and (18, 3, 0) layer 16,
# below 2^33, in a multiply pass at every table depth the tuner may pick: the
# products of twiddles of 64 + k and 32 + k bits.
@pytest.mark.parametrize("log_d,log_lanes,start", [(1, 4, 0), (5, 4, 0), (7, 6, 1), (12, 6, 1), (13, 4, 3),
                                                   (10, 6, 0), (9, 7, 2), (16, 6, 1), (14, 3, 2), (8, 3, 0),
                                                   (11, 4, 4), (12, 3, 1), (18, 3, 0)])
def test_ntt_matches_oracle(ctx, log_d, log_lanes, start):
    rng = np.random.default_rng(log_d * 7 + start)
    data = rng.integers(0, 2**63, (1 << (log_d + log_lanes)) * 2, dtype=np.uint64)
    data |= rng.integers(0, 2, data.shape, dtype=np.uint64) << np.uint64(63)
    d = to_dev(data)
    F.ntt(ctx, d, log_d, log_lanes, start)
    ref = O.ntt_interleaved(data, 1 << log_lanes, start)
    assert np.array_equal(host(d).view(np.uint64), ref)


@pytest.mark.parametrize("n,leaf", [(1, 1024), (2, 64), (8, 128), (64, 1024), (1024, 128), (32, 4096),
                                    (16, 2048), (4, 48), (2048, 1024)])
def test_merkle_matches_oracle(cuda_device, n, leaf):
    rng = np.random.default_rng(n + leaf)
    data = rng.integers(0, 256, n * leaf, dtype=np.uint8)
    tree = F.merkle_tree(to_dev(data), n, leaf)
    ref = O.merkle_tree(data, n)
    assert np.array_equal(host(tree).reshape(-1, 32), ref)


@pytest.mark.parametrize("n_log", [3, 6, 8])
def test_commit_matches_oracle(ctx, n_log):
    m = 14 + n_log
    blocks = O.compressions(n_log, 99 + n_log)
    z, _, _, _ = F.generate_witness(to_dev(blocks), len(blocks), n_log, want_ab=False, want_stripe=False)
    root, cw, tree = F.commit(ctx, z, m)
    oz, _, _, _ = O.witness(blocks, n_log, want_ab=False, want_stripe=False)
    oroot, ocw, otree = O.commit(oz, m, want_codeword=True, want_tree=True)
    assert np.array_equal(host(cw).view(np.uint64), ocw)
    assert np.array_equal(host(tree).reshape(-1, 32), otree)
    assert root == oroot


@pytest.mark.parametrize("rows_log", [8, 10])
def test_rate_quarter_256_columns_4k_leaves_matches_oracle(ctx, rows_log):
    """The kernel-microbench shape: 2^rows x 256 columns of uniform F128, rate 1/4
    (two replica layers, then the NTT), Merkle leaves of 256 x 16 B = 4 KiB (four
    BLAKE3 chunks merged, non-root)."""
    m = 7 + 8 + rows_log
    rng = np.random.default_rng(rows_log)
    z = rng.integers(0, 2**63, (1 << (m - 7)) * 2, dtype=np.uint64)
    z |= rng.integers(0, 2, z.shape, dtype=np.uint64) << np.uint64(63)
    root, cw, tree = F.commit(ctx, to_dev(z), m, log_inv_rate=2, log_batch_size=8)
    oroot, ocw, otree = O.commit(z, m, 2, 8, want_codeword=True, want_tree=True)
    assert np.array_equal(host(cw).view(np.uint64), ocw)
    assert np.array_equal(host(tree).reshape(-1, 32), otree)
    assert root == oroot


def test_ntt_autotuner_records_a_shape_and_keeps_results(ctx, monkeypatch):
    import ctypes
    L = F.lib()
    L.flock_ntt_tuned_variant.argtypes = [ctypes.c_int] * 4
    L.flock_ntt_tuned_table_end.argtypes = [ctypes.c_int] * 4
    rng = np.random.default_rng(5)
    data = rng.integers(0, 2**63, (1 << (15 + 4)) * 2, dtype=np.uint64)
    ref = O.ntt_interleaved(data, 16, 1)
    d = to_dev(data)
    F.ntt(ctx, d, 15, 4, 1)
    assert L.flock_ntt_tuned_variant(0, 15, 4, 1) in (0, 1, 2)
    # table passes of two layers from the start layer, ending where blocks
    # hold 2^8..2^10 quad-lanes (the tuned depth)
    te = L.flock_ntt_tuned_table_end(0, 15, 4, 1)
    assert (te - 1) % 2 == 0 and 1 <= te <= 15
    assert np.array_equal(host(d).view(np.uint64), ref)
    d = to_dev(data)
    F.ntt(ctx, d, 15, 4, 1)  # the tuned shape again: the same result
    assert np.array_equal(host(d).view(np.uint64), ref)
    # tuning off: the default shape, same result, nothing recorded
    monkeypatch.setenv("FLOCK_NTT_TUNE", "0")
    data2 = rng.integers(0, 2**63, (1 << (14 + 4)) * 2, dtype=np.uint64)
    d2 = to_dev(data2)
    F.ntt(ctx, d2, 14, 4, 1)
    assert L.flock_ntt_tuned_variant(0, 14, 4, 1) == -1
    assert np.array_equal(host(d2).view(np.uint64), O.ntt_interleaved(data2, 16, 1))


def test_merkle_autotuner_records_levels_and_keeps_the_tree(cuda_device, monkeypatch):
    import ctypes
    L = F.lib()
    L.flock_merkle_tuned_levels.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]
    rng = np.random.default_rng(12)
    n, leaf = 1 << 12, 64
    data = rng.integers(0, 256, n * leaf, dtype=np.uint8)
    ref = O.merkle_tree(data, n)
    tree = F.merkle_tree(to_dev(data), n, leaf)  # tuned here: every candidate writes the same tree
    assert L.flock_merkle_tuned_levels(0, n, leaf) in (0, 1, 2)
    assert np.array_equal(host(tree).reshape(-1, 32), ref)
    tree = F.merkle_tree(to_dev(data), n, leaf)  # the tuned level count
    assert np.array_equal(host(tree).reshape(-1, 32), ref)
    # tuning off: nothing recorded for a new shape, the same tree
    monkeypatch.setenv("FLOCK_MERKLE_TUNE", "0")
    data2 = rng.integers(0, 256, n * 32, dtype=np.uint8)
    tree2 = F.merkle_tree(to_dev(data2), n, 32)
    assert L.flock_merkle_tuned_levels(0, n, 32) == -1
    assert np.array_equal(host(tree2).reshape(-1, 32), O.merkle_tree(data2, n))


@pytest.mark.parametrize("variant", ["0", "1", "2"])
@pytest.mark.parametrize("log_d,log_lanes,start", [(13, 6, 2), (14, 5, 0), (15, 6, 1), (9, 7, 0)])
def test_ntt_every_pass_shape_matches_oracle(ctx, monkeypatch, variant, log_d, log_lanes, start):
    # each multiply-pass shape fixed in turn, on codes whose last pass is no
    # deeper than the shape's positions per thread (one thread per lane, 32
    # lanes per block) or deeper (two stages through the shared tile)
    monkeypatch.setenv("FLOCK_NTT_VARIANT", variant)
    rng = np.random.default_rng(log_d * 13 + log_lanes + int(variant))
    data = rng.integers(0, 2**63, (1 << (log_d + log_lanes)) * 2, dtype=np.uint64)
    d = to_dev(data)
    F.ntt(ctx, d, log_d, log_lanes, start)
    assert np.array_equal(host(d).view(np.uint64), O.ntt_interleaved(data, 1 << log_lanes, start))


# 64-lane codes whose table passes (default depth) end at layer log_d - 3, so
# the deep-table pass takes the last three layers: from no table pass (4, 1)
# to layer 13 of a 2^16-position transform.
@pytest.mark.parametrize("log_d,start", [(4, 1), (7, 0), (9, 0), (12, 1), (13, 2), (16, 1)])
def test_ntt_deep_table_pass_matches_oracle(ctx, monkeypatch, log_d, start):
    """The last three layers through per-block tables of the narrow twiddles'
    unreduced products (the pass shape FLOCK_NTT_VARIANT=3 fixes)."""
    monkeypatch.setenv("FLOCK_NTT_VARIANT", "3")
    rng = np.random.default_rng(log_d * 17 + start)
    data = rng.integers(0, 2**63, (1 << (log_d + 6)) * 2, dtype=np.uint64)
    data |= rng.integers(0, 2, data.shape, dtype=np.uint64) << np.uint64(63)
    d = to_dev(data)
    F.ntt(ctx, d, log_d, 6, start)
    assert np.array_equal(host(d).view(np.uint64), O.ntt_interleaved(data, 64, start))


def test_rate_quarter_256_columns_2e16_rows(ctx):
    """The kernel-microbench shape at its smallest stated size, 2^16 rows x 256
    columns (rate 1/4: 2^18 codeword positions, 1 GiB): columns are independent
    transforms, so three of them are checked against the oracle's one-column
    commit; the whole tree (4 KiB leaves) against the oracle's Merkle tree of
    the device codeword."""
    rows_log, cols_log = 16, 8
    m = 7 + cols_log + rows_log
    rng = np.random.default_rng(2016)
    z = rng.integers(0, 2**63, (1 << (m - 7)) * 2, dtype=np.uint64)
    z |= rng.integers(0, 2, z.shape, dtype=np.uint64) << np.uint64(63)
    root, cw, tree = F.commit(ctx, to_dev(z), m, log_inv_rate=2, log_batch_size=cols_log)
    cwb = host(cw)
    cwh = cwb.view(np.uint64).reshape(1 << (rows_log + 2), 1 << cols_log, 2)
    zc = z.reshape(1 << rows_log, 1 << cols_log, 2)
    for c in (0, 77, 255):
        _, ocw, _ = O.commit(np.ascontiguousarray(zc[:, c, :]).reshape(-1), 7 + rows_log, 2, 0, want_codeword=True)
        assert np.array_equal(np.ascontiguousarray(cwh[:, c, :]).reshape(-1), ocw), c
    otree = O.merkle_tree(cwb, 1 << (rows_log + 2))
    assert np.array_equal(host(tree).reshape(-1, 32), otree)
    assert root == otree[-1].tobytes()


def test_rate_quarter_256_columns_2e22_rows(ctx):
    """The kernel-microbench shape at its largest stated size, 2^22 rows x 256
    columns at rate 1/4 (2^24 codeword positions, a 64 GiB codeword): two
    columns against the oracle's one-column commit; the Merkle tree (4 KiB
    leaves) by sampled leaves against the oracle's leaf hash, every parent of
    the top eleven levels against the oracle's parent hash, and the root."""
    import torch
    rows_log, cols_log = 22, 8
    m = 7 + cols_log + rows_log
    n_pos = 1 << (rows_log + 2)
    g = torch.Generator(device="cuda").manual_seed(2022)
    z = torch.randint(-2**62, 2**62, ((1 << (m - 7)) * 2,), dtype=torch.int64, device="cuda", generator=g)
    root, cw, tree = F.commit(ctx, z.view(torch.uint8), m, log_inv_rate=2, log_batch_size=cols_log)
    torch.cuda.synchronize()
    zc = z.view(1 << rows_log, 1 << cols_log, 2)
    cwc = cw.view(torch.int64).view(n_pos, 1 << cols_log, 2)
    for c in (3, 200):
        col = zc[:, c, :].contiguous().cpu().numpy().view(np.uint64).reshape(-1)
        _, ocw, _ = O.commit(col, 7 + rows_log, 2, 0, want_codeword=True)
        assert np.array_equal(cwc[:, c, :].contiguous().cpu().numpy().view(np.uint64).reshape(-1), ocw), c
        del ocw
    t = tree.view(-1, 32)
    rng = np.random.default_rng(22)
    for leaf in [0, n_pos - 1] + [int(x) for x in rng.integers(0, n_pos, 30)]:
        data = cw[leaf * 4096:(leaf + 1) * 4096].cpu().numpy()
        assert O.leaf_cv(data) == t[leaf].cpu().numpy().tobytes(), leaf
    # flat tree: level k (2^(24-k) nodes) starts at 2^25 - 2^(25-k)
    starts = [(1 << 25) - (1 << (25 - k)) for k in range(25)]
    for k in range(13, 24):
        below = t[starts[k]:starts[k] + (1 << (24 - k))].cpu().numpy()
        above = t[starts[k + 1]:starts[k + 1] + (1 << (23 - k))].cpu().numpy()
        assert np.array_equal(O.parent_cvs(below), above), k
    assert root == t[-1].cpu().numpy().tobytes()
    del z, cw, tree
    torch.cuda.empty_cache()

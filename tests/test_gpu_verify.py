"""The device-accelerated verifier (flock_verify): accepts the prover's and
the oracle's proofs, rejects tampered and malformed bundles."""
import numpy as np
import pytest

import flock_challenge_gb300 as F
import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def proof10(cuda_device):
    return F.Blake3Setup(1 << 10).prove_seed(3)


@pytest.mark.parametrize("log2,seed", [(8, 1), (9, 7), (12, 2)])
def test_gpu_proofs_verify(cuda_device, log2, seed):
    p = F.Blake3Setup(1 << log2).prove_seed(seed)
    assert F.verify(p)


def test_oracle_proof_verifies_and_oracle_accepts_the_same(cuda_device):
    blocks = O.compressions(8, 21)[:200]
    p = O.prove(blocks, 8)
    assert F.verify(p)
    assert O.verify(p, 22)[0]


def test_tampered_proofs_rejected(proof10):
    assert F.verify(proof10)
    n = len(proof10)
    rng = np.random.default_rng(1)
    # header/params, zerocheck, lincheck, ring switch and Ligerito regions
    offsets = [60, 100, 2100, 2600, 4300, 5000] + sorted(int(x) for x in rng.integers(6000, n - 8, 24))
    for off in offsets:
        b = bytearray(proof10)
        b[off] ^= 0x10
        assert not F.verify(bytes(b)), off


def test_truncated_and_extended_rejected(proof10):
    assert not F.verify(proof10[:-1])
    assert not F.verify(proof10 + b"\0")
    assert not F.verify(proof10[:1000])
    assert not F.verify(b"")


def test_batch(proof10):
    bad = bytearray(proof10)
    bad[-20] ^= 1
    assert F.verify_batch([proof10, bytes(bad), proof10]) == [True, False, True]


def test_ranked_size_proof_verifies(cuda_device):
    import time
    s = F.Blake3Setup(1 << 18)
    p = s.prove_seed(11)
    F.verify(p)  # warm (statement digest, device buffers)
    t = time.perf_counter()
    assert F.verify(p)
    assert time.perf_counter() - t < 5.0
    b = bytearray(p)
    b[len(b) // 2] ^= 4
    assert not F.verify(bytes(b))


def test_every_supported_size_proves_and_verifies(cuda_device):
    """m = 22 .. 35 (2^8 .. 2^21 compressions): every Ligerito configuration."""
    for log2 in range(8, 22):
        p = F.Blake3Setup(1 << log2).prove_seed(1000 + log2)
        assert F.verify(p), log2
        assert len(p) < 500_000
        if log2 in (17, 19):  # both byte-table splits of the Ligerito basis, checked by the oracle verifier
            ok, why = O.verify(p, 14 + log2)
            assert ok, (log2, why)


def test_ragged_large_input_verifies(cuda_device):
    import torch
    n = 100_000
    d = F.generate_inputs(17, 5)
    blocks = np.frombuffer(d.cpu().numpy().tobytes(), dtype=F.COMPRESSION_DTYPE)[:n].copy()
    p = F.Blake3Setup(n).prove_fast(blocks)
    assert F.verify(p)
    torch.cuda.synchronize()

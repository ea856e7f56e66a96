"""The prove_fast seam (crates/flock-prover/src/r1cs_hashes/blake3.rs:3405-3409):
a caller-owned Fiat-Shamir transcript handle (flock_transcript_*) and the
proof, commitment root and R1csClaim of flock_prove_challenger.

The transcript is host code, so its test runs without a GPU; the prove and
verify tests are marked gpu.
"""
import pytest

import flock_challenge_gb300 as F
import oracle_lib as O

DOMAIN = b"caller-domain\x00v7"  # a non-default domain, with a NUL byte


def drive(t):
    """The same prefix of Challenger calls on either transcript (challenger.rs:34-110)."""
    t.observe_label(b"outer-protocol")
    t.observe_bytes(bytes(range(40)))
    t.observe_f128((0x0123456789ABCDEF, 0xFEDCBA9876543210))
    t.observe_f128_slice([(i, 3 * i + 1) for i in range(5)])
    t.observe_f128_slice([])
    a = t.sample_f128()
    v = t.sample_f128_vec(3)
    t.observe_label(b"")
    return a, v


def test_transcript_handle_matches_oracle_transcript():
    mine, ref = F.FsChallenger(DOMAIN), O.Transcript(DOMAIN)
    assert drive(mine) == drive(ref)
    # fork: independent copies that stay in lockstep with the original
    f1, f2 = mine.fork(), ref.fork()
    assert f1.sample_f128() == f2.sample_f128()
    assert mine.sample_f128_vec(0) == ref.sample_f128_vec(0)
    assert mine.sample_f128() == ref.sample_f128() != f1.sample_f128()
    # the vector squeeze is not n single samples (FsChallenger's own form)
    g = F.FsChallenger(DOMAIN)
    h = g.fork()
    assert g.sample_f128_vec(2) != [h.sample_f128(), h.sample_f128()]


@pytest.mark.gpu
def test_prove_with_caller_transcript_matches_oracle(cuda_device):
    n_log = 8
    blocks = O.compressions(n_log, 21)
    mine, ref = F.FsChallenger(DOMAIN), O.Transcript(DOMAIN)
    drive(mine)
    drive(ref)
    setup = F.Blake3Setup(1 << n_log)
    before = mine.fork()
    proof, root, claim = setup.prove_fast(blocks, challenger=mine)
    oproof, oroot, oclaim = O.prove_with(blocks, n_log, ref)
    assert proof == oproof
    assert root == oroot
    assert claim == oclaim
    assert len(claim["ab"]["x_outer"]) == n_log and len(claim["c"]["x_inner_rest"]) == 8
    # the transcripts leave the proof in the same state
    assert mine.sample_f128() == ref.sample_f128()
    # a different prefix gives a different proof; the default entry differs too
    assert proof != setup.prove_fast(blocks)
    # the verifier replays from the same prefix, and only from it
    ok_t = before.fork()
    assert F.verify(proof, challenger=ok_t)
    okr, why = O.verify_with(proof, 14 + n_log, _prefixed())
    assert okr, why
    assert not F.verify(proof, challenger=F.FsChallenger(DOMAIN))
    assert not F.verify(proof)  # the benchmark domain without the prefix


def _prefixed():
    t = O.Transcript(DOMAIN)
    drive(t)
    return t


@pytest.mark.gpu
def test_prove_challenger_leaves_transcript_unchanged_on_small_buffer(cuda_device):
    import ctypes
    import numpy as np
    n_log = 8
    blocks = O.compressions(n_log, 22)
    setup = F.Blake3Setup(1 << n_log)
    t = F.FsChallenger(DOMAIN)
    probe = t.fork()
    L = F._proto_lib()
    small = np.zeros(16, np.uint8)
    ln = ctypes.c_size_t()
    rc = L.flock_prove_challenger(setup.ctx.handle, blocks.ctypes.data_as(ctypes.c_void_p), len(blocks), 0,
                                  t.handle, small.ctypes.data_as(ctypes.c_void_p), small.size, ctypes.byref(ln),
                                  None, None)
    assert rc == -5 and ln.value > 200_000
    assert t.fork().sample_f128() == probe.fork().sample_f128()  # unchanged
    p1, _, _ = setup.prove_fast(blocks, challenger=t)
    p2, _, _ = setup.prove_fast(blocks, challenger=probe)
    assert p1 == p2

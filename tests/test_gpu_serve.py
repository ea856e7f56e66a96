"""Batched and served proving: every proof equals the plain path's proof,
alone and in the mix, and the device-memory budget is respected."""
import time

import numpy as np
import pytest

import flock_challenge_gb300 as F
import oracle_lib as O

pytestmark = pytest.mark.gpu


def plain(log2, seed):
    return F.Blake3Setup(1 << log2).prove_seed(seed)


def test_batch_matches_plain_path(cuda_device):
    sizes, seeds = [8, 10, 9, 8, 11], [3, 1, 4, 1, 5]
    with F.Server(workers=3) as srv:
        proofs = srv.prove_batch(sizes, seeds)
    for l, sd, p in zip(sizes, seeds, proofs):
        assert p == plain(l, sd), (l, sd)
    # and the smallest against the oracle
    blocks = O.compressions(8, 3)
    assert proofs[0] == O.prove(blocks, 8)


def test_server_requests_same_alone_and_in_the_mix(cuda_device):
    reqs = [(10, 7), (8, 9), (9, 11), (8, 13), (11, 2), (8, 9)]
    alone = {r: plain(*r) for r in set(reqs)}
    with F.Server(workers=3) as srv:
        ids = [srv.submit_seed(l, s) for l, s in reqs]
        got = [srv.wait(i) for i in ids]
    for r, p in zip(reqs, got):
        assert p == alone[r], r


def test_server_host_inputs(cuda_device):
    blocks = O.compressions(9, 77)[:300]
    want = F.Blake3Setup(300).prove_fast(blocks)
    with F.Server(workers=2) as srv:
        rid = srv.submit(blocks)
        p = None
        while p is None:
            p = srv.poll(rid)
            time.sleep(0.005)
    assert p == want


def test_server_budget_admission(cuda_device):
    budget = F.footprint_bytes(9) + F.footprint_bytes(8) // 2
    with F.Server(workers=3, hbm_budget=budget) as srv:
        ids = [srv.submit_seed(9, s) for s in range(4)]
        peak = 0
        done = {}
        while len(done) < len(ids):
            peak = max(peak, srv.reserved_bytes())
            for i in ids:
                if i not in done:
                    p = srv.poll(i)
                    if p is not None:
                        done[i] = p
            time.sleep(0.002)
        assert peak <= budget
        with pytest.raises(F.FlockError, match="out of memory"):
            srv.submit_seed(14, 0)
    for s, i in enumerate(ids):
        assert done[i] == plain(9, s)


def test_context_budget_rejects_large_proof(cuda_device):
    ctx = F.Blake3Setup(1 << 10)
    ctx.ctx = F.Context(0, hbm_budget=F.footprint_bytes(9))
    with pytest.raises(F.FlockError, match="out of memory"):
        ctx.prove_seed(1)


@pytest.mark.parametrize("log2", [8, 10, 12])
def test_footprint_bounds_what_a_prover_holds(cuda_device, log2):
    with F.Server(workers=1) as srv:
        srv.wait(srv.submit_seed(log2, 1))
        # a worker's reservation is max(estimate, bytes actually held)
        assert srv.reserved_bytes() == F.footprint_bytes(log2)

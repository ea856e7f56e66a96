"""Hash-chain proofs on the GPU (flock_prove_chain / flock_verify_chain)
against the oracle: byte-identical bundles, verifier agreement both ways,
the reference's rejections, and at 2^18 steps the size-independent checks
(the chain bundle's R1CS sections equal the plain proof's under the same
transcript domain, and the bundle verifies)."""
import numpy as np
import pytest

import flock_challenge_gb300 as F
import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("steps,seed,cv0,domain", [
    (256, 0, None, None),
    (512, 0xB35113E, np.arange(1, 9, dtype=np.uint32) * 0x01010101, None),
    (1024, 7, None, b"b3-chain-lig"),
])
def test_chain_bundle_matches_oracle(cuda_device, steps, seed, cv0, domain):
    blocks = F.chain_inputs(steps, seed, cv0)
    want = O.prove_chain(blocks, domain or b"flock_chain-cli")
    got = F.Blake3Setup(steps).prove_chain(blocks, domain)
    assert got[:7] == b"FLOCK\x04\x03"
    assert len(got) == len(want)
    assert got == want
    assert F.verify_chain(got, domain)
    assert O.verify_chain(got, domain or b"flock_chain-cli")[0]


def test_chain_rejections(cuda_device):
    blocks = F.chain_inputs(256, 0xB31234)
    setup = F.Blake3Setup(256)
    bundle = setup.prove_chain(blocks)
    assert F.verify_chain(bundle)
    for off in (len(bundle) - 2 * 264 + 8 + 5, len(bundle) - 1):  # a cv_0 bit, a cv_last bit
        b = bytearray(bundle)
        b[off] ^= 1
        assert not F.verify_chain(bytes(b)), off
    assert not F.verify_chain(bundle, b"b3-chain")
    assert not F.verify_chain(bundle[:-1])
    assert not F.verify_chain(bundle + b"\x00")
    # tampered messages: a zerocheck value, a shift-sumcheck value, an opening byte
    for off in (200, len(bundle) // 2, len(bundle) - 600):
        b = bytearray(bundle)
        b[off] ^= 0x10
        assert not F.verify_chain(bytes(b)), off
    # a broken link (instance 2 does not follow instance 1), proven as is
    broken = blocks.copy()
    broken["cv"][2] = np.arange(8, dtype=np.uint32) * 977
    bb = setup.prove_chain(broken)
    assert bb == O.prove_chain(broken)
    assert not F.verify_chain(bb)
    # R1CS bundles are not chain bundles and vice versa
    assert not F.verify_chain(setup.prove_fast(blocks))
    assert not F.verify(bundle)


def test_chain_requires_full_power_of_two(cuda_device):
    blocks = F.chain_inputs(300, 1)
    ctx = F.Context(0)
    L = F._proto_lib()
    import ctypes
    buf = np.zeros(1 << 20, np.uint8)
    ln = ctypes.c_size_t()
    rc = L.flock_prove_chain(ctx.handle, blocks.ctypes.data_as(ctypes.c_void_p), 300, None,
                             buf.ctypes.data_as(ctypes.c_void_p), buf.size, ctypes.byref(ln))
    assert rc == -1  # FLOCK_ERR_SHAPE: steps must be 2^k >= 2^8
    rc = L.flock_prove_chain(ctx.handle, blocks.ctypes.data_as(ctypes.c_void_p), 128, None,
                             buf.ctypes.data_as(ctypes.c_void_p), buf.size, ctypes.byref(ln))
    assert rc == -1


def _sections(bundle, chain):
    """(root, zerocheck + lincheck bytes) of a bundle: fixed-size sections at m = 32."""
    m = 32
    o = 7 + (4 if chain else 0)
    root = bundle[o:o + 32]
    o += 32 + 8 * 3 + 4 * 2
    zc = 2 * (8 + 64 * 16) + 8 + (m - 6) * 32 + 3 * 16
    lc = 8 + 8 * 32 + 8 + 64 * 16
    return root, bundle[o:o + zc + lc]


def test_chain_full_size(cuda_device):
    steps = 1 << 18
    blocks = F.chain_inputs(steps, 42)
    setup = F.Blake3Setup(steps)
    bundle = setup.prove_chain(blocks, b"flock-bench-v0")
    assert F.verify_chain(bundle, b"flock-bench-v0")
    plain = setup.prove_fast(blocks)
    # same witness, same transcript up to the end of lincheck
    assert _sections(bundle, True) == _sections(plain, False)
    # and a second proof of the same chain is byte-identical
    assert setup.prove_chain(blocks, b"flock-bench-v0") == bundle

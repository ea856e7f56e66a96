"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure: used by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py only. Builds the oracle with make on first use.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

_lock = threading.Lock()
_lib = None

COMP_DTYPE = np.dtype([("cv", "<u4", 8), ("m", "<u4", 16), ("counter", "<u8"),
                       ("block_len", "<u4"), ("flags", "<u4")])


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "-j8"], check=True)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            P = ctypes.c_void_p
            sz = ctypes.c_size_t
            L.oracle_generate_compressions.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, P]
            L.oracle_compression_size.restype = sz
            L.oracle_witness.argtypes = [P, sz, ctypes.c_int, P, P, P, P]
            L.oracle_statement_digest.argtypes = [ctypes.c_int, P]
            L.oracle_matrices.argtypes = [P, P, P]
            L.oracle_matrices.restype = sz
            L.oracle_ntt_twiddles.argtypes = [ctypes.c_int, P]
            L.oracle_ntt_interleaved.argtypes = [P, sz, sz, ctypes.c_int]
            L.oracle_merkle_tree.argtypes = [P, sz, sz, P]
            L.oracle_commit.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P]
            L.oracle_gf_mul.argtypes = [P, P, P]
            L.oracle_gf_inv.argtypes = [P, P]
            L.oracle_phi8.argtypes = [ctypes.c_uint8, P]
            L.oracle_gf8_mul.argtypes = [ctypes.c_uint8, ctypes.c_uint8]
            L.oracle_gf8_mul.restype = ctypes.c_uint8
            L.oracle_b3_compress.argtypes = [P, P, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, P]
            L.oracle_b3_hash.argtypes = [P, sz, P]
            L.oracle_b3_xof.argtypes = [P, sz, P, sz]
            L.oracle_leaf_cv.argtypes = [P, sz, P]
            assert L.oracle_compression_size() == COMP_DTYPE.itemsize
            _lib = L
    return _lib


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def gf_mul(a, b):
    out = np.zeros(2, np.uint64)
    lib().oracle_gf_mul(ptr(np.array(a, np.uint64)), ptr(np.array(b, np.uint64)), ptr(out))
    return (int(out[0]), int(out[1]))


def gf_inv(a):
    out = np.zeros(2, np.uint64)
    lib().oracle_gf_inv(ptr(np.array(a, np.uint64)), ptr(out))
    return (int(out[0]), int(out[1]))


def phi8(v):
    out = np.zeros(2, np.uint64)
    lib().oracle_phi8(v, ptr(out))
    return (int(out[0]), int(out[1]))


def compressions(log2_size, seed, canary=False):
    out = np.zeros(1 << log2_size, COMP_DTYPE)
    lib().oracle_generate_compressions(log2_size, seed, int(canary), ptr(out))
    return out


def witness(blocks, n_blocks_log, want_ab=True, want_stripe=True):
    m = 14 + n_blocks_log
    n128 = 1 << (m - 7)
    z = np.zeros(2 * n128, np.uint64)
    a = np.zeros(2 * n128, np.uint64) if want_ab else None
    b = np.zeros(2 * n128, np.uint64) if want_ab else None
    s = np.zeros((1 << m) // 8, np.uint8) if want_stripe else None
    blocks = np.ascontiguousarray(blocks)
    lib().oracle_witness(ptr(blocks), len(blocks), n_blocks_log, ptr(z), ptr(a), ptr(b), ptr(s))
    return z, a, b, s


def statement_digest(m):
    out = np.zeros(32, np.uint8)
    lib().oracle_statement_digest(m, ptr(out))
    return out.tobytes()


def matrices():
    a_len = np.zeros(1 << 14, np.uint32)
    b_len = np.zeros(1 << 14, np.uint32)
    nnz = lib().oracle_matrices(ptr(a_len), ptr(b_len), None)
    cols = np.zeros(nnz, np.uint32)
    lib().oracle_matrices(ptr(a_len), ptr(b_len), ptr(cols))
    return a_len, b_len, cols


def ntt_twiddles(dim):
    out = np.zeros(2 * ((1 << dim) - 1), np.uint64)
    lib().oracle_ntt_twiddles(dim, ptr(out))
    return out


def ntt_interleaved(data_u64, num_ntts, start_layer):
    d = np.ascontiguousarray(data_u64, dtype=np.uint64).copy()
    lib().oracle_ntt_interleaved(ptr(d), d.size // 2, num_ntts, start_layer)
    return d


def merkle_tree(data_u8, n_leaves):
    d = np.ascontiguousarray(data_u8, dtype=np.uint8)
    out = np.zeros(32 * (2 * n_leaves - 1), np.uint8)
    lib().oracle_merkle_tree(ptr(d), d.size, n_leaves, ptr(out))
    return out.reshape(-1, 32)


def commit(z_u64, m, log_inv_rate=1, log_batch_size=6, want_codeword=False, want_tree=False):
    root = np.zeros(32, np.uint8)
    n_pos = 1 << (m - 7 - log_batch_size + log_inv_rate)
    cw = np.zeros(2 * n_pos * (1 << log_batch_size), np.uint64) if want_codeword else None
    tree = np.zeros(32 * (2 * n_pos - 1), np.uint8) if want_tree else None
    z = np.ascontiguousarray(z_u64, dtype=np.uint64)
    lib().oracle_commit(ptr(z), m, log_inv_rate, log_batch_size, ptr(root), ptr(cw), ptr(tree))
    return root.tobytes(), cw, (tree.reshape(-1, 32) if tree is not None else None)


def b3_compress(cv, block, counter, block_len, flags):
    out = np.zeros(16, np.uint32)
    lib().oracle_b3_compress(ptr(np.array(cv, np.uint32)), ptr(np.array(block, np.uint32)),
                             counter, block_len, flags, ptr(out))
    return out


def b3_hash(data):
    d = np.frombuffer(bytes(data), np.uint8).copy() if len(data) else np.zeros(1, np.uint8)
    out = np.zeros(32, np.uint8)
    lib().oracle_b3_hash(ptr(d), len(data), ptr(out))
    return out.tobytes()


def b3_xof(data, n):
    d = np.frombuffer(bytes(data), np.uint8).copy() if len(data) else np.zeros(1, np.uint8)
    out = np.zeros(n, np.uint8)
    lib().oracle_b3_xof(ptr(d), len(data), ptr(out), n)
    return out.tobytes()


def leaf_cv(data):
    d = np.frombuffer(bytes(data), np.uint8).copy()
    out = np.zeros(32, np.uint8)
    lib().oracle_leaf_cv(ptr(d), len(data), ptr(out))
    return out.tobytes()


def parent_cvs(children_u8):
    """Parent chaining values (BLAKE3 PARENT nodes) of consecutive node pairs."""
    c = np.ascontiguousarray(children_u8, dtype=np.uint8).reshape(-1)
    n = c.size // 64
    out = np.zeros(32 * n, np.uint8)
    L = lib()
    L.oracle_parent_cvs.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    L.oracle_parent_cvs(ptr(c), n, ptr(out))
    return out.reshape(-1, 32)


def _proto():
    L = lib()
    if not getattr(L, "_proto_ready", False):
        P = ctypes.c_void_p
        L.oracle_prove.argtypes = [P, ctypes.c_size_t, ctypes.c_int, P, ctypes.c_size_t,
                                   ctypes.POINTER(ctypes.c_size_t)]
        L.oracle_verify.argtypes = [P, ctypes.c_size_t, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_chain_inputs.argtypes = [ctypes.c_size_t, ctypes.c_uint64, P, P]
        L.oracle_prove_chain.argtypes = [P, ctypes.c_size_t, ctypes.c_int, ctypes.c_char_p, P, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_size_t)]
        L.oracle_verify_chain.argtypes = [P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_shift_mle.argtypes = [P, P, ctypes.c_int, P]
        L.oracle_f8_extend_ntt.argtypes = [ctypes.c_uint64, P]
        L.oracle_f8_extend_lagrange.argtypes = [ctypes.c_uint64, P]
        L.oracle_warm.argtypes = [ctypes.c_int]
        L._proto_ready = True
    return L


def prove(blocks, n_blocks_log):
    """Full oracle proof; returns the wire bytes."""
    L = _proto()
    blocks = np.ascontiguousarray(blocks)
    cap = 4_000_000
    out = np.zeros(cap, np.uint8)
    ln = ctypes.c_size_t()
    rc = L.oracle_prove(ptr(blocks), len(blocks), n_blocks_log, ptr(out), cap, ctypes.byref(ln))
    assert rc == 0, rc
    return out[:ln.value].tobytes()


def warm(m):
    """Builds the oracle's cached setup (matrices, statement digest) for m."""
    _proto().oracle_warm(m)


def uses_pmull():
    """True when the oracle's GF(2^128) product runs on the Arm PMULL instruction."""
    return bool(lib().oracle_gf_uses_pmull())


def verify(proof_bytes, m):
    """Oracle verifier: returns (accepted, reason)."""
    L = _proto()
    buf = np.frombuffer(proof_bytes, np.uint8).copy()
    why = ctypes.create_string_buffer(256)
    rc = L.oracle_verify(ptr(buf), len(proof_bytes), m, why, 256)
    return rc == 0, why.value.decode()


def chain_inputs(steps, seed, cv0=None):
    """Honest BLAKE3 chain (the flock_chain CLI's generator): each cv is the
    previous compression's first 8 output words; cv0 None = the BLAKE3 IV."""
    L = _proto()
    out = np.zeros(steps, COMP_DTYPE)
    c = None if cv0 is None else ptr(np.ascontiguousarray(cv0, dtype=np.uint32))
    L.oracle_chain_inputs(steps, seed, c, ptr(out))
    return out


def prove_chain(blocks, domain=b"flock_chain-cli"):
    """Oracle chain proof (ChainProofBundleLigerito bytes) of 2^k compressions."""
    L = _proto()
    blocks = np.ascontiguousarray(blocks)
    n_log = int(len(blocks)).bit_length() - 1
    cap = 4_000_000
    out = np.zeros(cap, np.uint8)
    ln = ctypes.c_size_t()
    rc = L.oracle_prove_chain(ptr(blocks), len(blocks), n_log, domain, ptr(out), cap, ctypes.byref(ln))
    assert rc == 0, rc
    return out[:ln.value].tobytes()


def verify_chain(proof_bytes, domain=b"flock_chain-cli"):
    """Oracle chain verifier: returns (accepted, reason)."""
    L = _proto()
    buf = np.frombuffer(proof_bytes, np.uint8).copy()
    why = ctypes.create_string_buffer(256)
    rc = L.oracle_verify_chain(ptr(buf), len(proof_bytes), domain, why, 256)
    return rc == 0, why.value.decode()


def shift_mle(a, b):
    """shift(a, b) for points given as lists of (lo, hi) u64 pairs."""
    L = _proto()
    x = np.array(a, dtype=np.uint64).reshape(-1)
    y = np.array(b, dtype=np.uint64).reshape(-1)
    out = np.zeros(2, np.uint64)
    L.oracle_shift_mle(ptr(x), ptr(y), len(a), ptr(out))
    return int(out[0]), int(out[1])


def f8_extend(row, via="ntt"):
    L = _proto()
    out = np.zeros(64, np.uint8)
    (L.oracle_f8_extend_ntt if via == "ntt" else L.oracle_f8_extend_lagrange)(row, ptr(out))
    return out


class Transcript:
    """The oracle's FsChallenger restatement (challenger.rs:183-438) behind a
    handle, mirroring flock_challenge_gb300.FsChallenger's methods."""

    def __init__(self, domain=b"flock-bench-v0", _h=None):
        L = _tr_lib()
        self._h = _h if _h is not None else L.oracle_transcript_new(domain, len(domain))

    def fork(self):
        return Transcript(_h=_tr_lib().oracle_transcript_clone(self._h))

    def observe_label(self, b):
        _tr_lib().oracle_transcript_label(self._h, bytes(b), len(b))

    def observe_f128(self, v):
        _tr_lib().oracle_transcript_observe_f128(self._h, ptr(np.array(v, np.uint64)))

    def observe_f128_slice(self, vs):
        a = np.array(vs, np.uint64).reshape(-1) if len(vs) else np.zeros(2, np.uint64)
        _tr_lib().oracle_transcript_observe_slice(self._h, ptr(a), len(vs))

    def observe_bytes(self, b):
        _tr_lib().oracle_transcript_observe_bytes(self._h, bytes(b), len(b))

    def sample_f128(self):
        out = np.zeros(2, np.uint64)
        _tr_lib().oracle_transcript_sample(self._h, ptr(out))
        return int(out[0]), int(out[1])

    def sample_f128_vec(self, n):
        out = np.zeros(2 * max(n, 1), np.uint64)
        _tr_lib().oracle_transcript_sample_vec(self._h, n, ptr(out))
        return [(int(out[2 * i]), int(out[2 * i + 1])) for i in range(n)]

    def __del__(self):
        try:
            _tr_lib().oracle_transcript_free(self._h)
        except Exception:
            pass


def _tr_lib():
    L = _proto()
    if not getattr(L, "_tr_ready", False):
        P = ctypes.c_void_p
        L.oracle_transcript_new.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_transcript_new.restype = P
        L.oracle_transcript_clone.argtypes = [P]
        L.oracle_transcript_clone.restype = P
        L.oracle_transcript_free.argtypes = [P]
        L.oracle_transcript_label.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_transcript_observe_f128.argtypes = [P, P]
        L.oracle_transcript_observe_slice.argtypes = [P, P, ctypes.c_size_t]
        L.oracle_transcript_observe_bytes.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_transcript_sample.argtypes = [P, P]
        L.oracle_transcript_sample_vec.argtypes = [P, ctypes.c_size_t, P]
        L.oracle_prove_tr.argtypes = [P, ctypes.c_size_t, ctypes.c_int, P, P, ctypes.c_size_t,
                                      ctypes.POINTER(ctypes.c_size_t), P]
        L.oracle_verify_tr.argtypes = [P, ctypes.c_size_t, ctypes.c_int, P, ctypes.c_char_p, ctypes.c_size_t]
        L._tr_ready = True
    return L


def prove_with(blocks, n_blocks_log, transcript):
    """Oracle proof continuing `transcript` (advanced by the call). Returns
    (bundle bytes, root bytes, claim dict shaped as the GPU binding's)."""
    L = _tr_lib()
    blocks = np.ascontiguousarray(blocks)
    out = np.zeros(4_000_000, np.uint8)
    ln = ctypes.c_size_t()
    n_out = n_blocks_log  # m - 14
    claim = np.zeros(2 * (4 + 16 + 2 * n_out), np.uint64)
    rc = L.oracle_prove_tr(ptr(blocks), len(blocks), n_blocks_log, transcript._h, ptr(out), out.size,
                           ctypes.byref(ln), ptr(claim))
    assert rc == 0, rc
    f = [(int(claim[2 * i]), int(claim[2 * i + 1])) for i in range(claim.size // 2)]
    ab_inner, ab_outer = f[4:12], f[12:12 + n_out]
    c_inner, c_outer = f[12 + n_out:20 + n_out], f[20 + n_out:20 + 2 * n_out]
    cl = {"ab": {"z_skip": f[0], "x_inner_rest": ab_inner, "x_outer": ab_outer, "value": f[1]},
          "c": {"z_skip": f[2], "x_inner_rest": c_inner, "x_outer": c_outer, "value": f[3]}}
    bundle = out[:ln.value].tobytes()
    return bundle, bundle[7:39], cl


def verify_with(proof_bytes, m, transcript):
    """Oracle verifier continuing `transcript`: (accepted, reason)."""
    L = _tr_lib()
    buf = np.frombuffer(proof_bytes, np.uint8).copy()
    why = ctypes.create_string_buffer(256)
    rc = L.oracle_verify_tr(ptr(buf), len(proof_bytes), m, transcript._h, why, 256)
    return rc == 0, why.value.decode()
